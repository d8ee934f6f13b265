"""Benchmark of the batched hydroelastic contact step on GB300.

python bench.py --gpus N --steps K --warmup W [--impl reference]

Workload: 4096 independent tactile scenes (rigid 8x8 cm plate with a 16x16
taxel grid pressed by a soft sphere / ellipsoid / cylinder of 2k-8k tets, E in
5e4-5e5 Pa, penetration 0-4 mm, in-plane offset +-2 cm, velocities U[-0.1,0.1])
per GPU: the distribution the differentiable batched workload is defined on.
One step = the pair dispatch frames, LBVH broadphase, clipping, quadrature,
Hunt-Crossley + friction, per-pair wrench, taxel binning for all scenes, and
(when built) the adjoint.  Synthetic seeded inputs (no dataset exists).

The default arm runs the engine through its C ABI; `--impl reference` times
the CPU path (the FP64 restatement in oracle/, OpenMP over pairs) on a
bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "contact pairs/s fwd+adjoint, batched vs plain GPU path at 1e-5 rel wrench err"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--scenes", type=int, default=4096)
    ap.add_argument("--cpu-sample", type=int, default=256, help="scenes in the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(n_scenes, rank):
    from mujoco_contact_surfaces_gb300 import scenes
    return scenes.tactile(n_scenes, seed=scenes.SEED_ADJOINT + rank, velocities=True)


def config_dict(args, world, extra=None):
    c = {"workload": "tactile batched: 4096 scenes/GPU, rigid 8x8 cm plate + 16x16 taxels (5x5 rays/cell) "
                     "vs soft sphere/ellipsoid/cylinder 2k-8k tets",
         "scenes_per_gpu": args.scenes, "pairs_per_scene": 1, "representation": "kTriangle",
         "l2": "flushed between timed steps (256 MiB write)", "parallelism": f"scene shards x{world}"}
    if extra:
        c.update(extra)
    return c


def cpu_baseline(n_sample, rank, reps=3):
    """FP64 oracle, OpenMP over pairs, all host cores, on a bounded sample."""
    import oracle
    s = workload(n_sample, rank)
    o = oracle.Oracle(s)
    o.collide()  # warm
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        o.collide()
        ts.append(time.perf_counter() - t0)
    o.close()
    t = statistics.median(ts)
    return {"value": n_sample / t, "unit": "pairs/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"{n_sample} scenes of the same workload (1 pair + 1 sensor each), median of {reps}"}


class Clocks:
    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_{os.getpid()}.csv")

    def start(self):
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def algorithmic_bytes(eng, n_pair, n_sensor_pairs):
    """Sec. 8(d) bytes of one forward step: 80 B per distinct soft tet and 48 B
    per distinct rigid triangle with a non-empty polygon, 96 B of poses and
    48 B of wrench per pair, 1024 B of taxels per sensor pair."""
    eng.set_debug(1)
    eng.step()
    cand = eng.candidates()
    eng.set_debug(0)
    tets = len({(int(r[0]), int(r[1])) for r in cand})
    tris = len({(int(r[0]), int(r[2])) for r in cand if r[2] >= 0})
    narrow = 80 * tets + 48 * tris
    step = narrow + (96 + 48) * n_pair + 1024 * n_sensor_pairs
    return narrow, step, tets, tris, len(cand)


def run_gb300(args):
    import torch
    from mujoco_contact_surfaces_gb300 import scenes
    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))

    s = workload(args.scenes, rank)
    n_pair = len(s.g1)
    eng = scenes.build_engine(s, device=local)
    eng.enable_timing(True)
    narrow_bytes, step_bytes, n_tets, n_tris, n_poly = algorithmic_bytes(eng, n_pair, len(s.sensors))

    stream = torch.cuda.ExternalStream(eng.stream(), device=local)
    dev = torch.device("cuda", local)
    xpos = torch.tensor(s.xpos, dtype=torch.float64, device=dev)
    xmat = torch.tensor(s.xmat, dtype=torch.float64, device=dev)
    vel = torch.tensor(s.vel, dtype=torch.float64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    n_geom = s.n_geom
    torch.cuda.synchronize()

    def device_step():
        eng.set_poses_device(n_geom, xpos.data_ptr(), xmat.data_ptr(), vel.data_ptr())
        eng.step()

    for _ in range(args.warmup):
        device_step()
    eng.wrenches()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()

    clocks = Clocks(local)
    clocks.start()
    step_ms, narrow_ms = [], []
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1)
            e0.record(stream)
        device_step()
        with torch.cuda.stream(stream):
            e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        tm = eng.timings()
        narrow_ms.append(tm.ms_narrowphase)
    torch.cuda.synchronize()
    clk = clocks.stop()
    t_step = sum(step_ms) / len(step_ms)
    if world > 1:
        t = torch.tensor([t_step], dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_step = float(t[0])
    value = n_pair * world / (t_step * 1e-3)

    # end to end through the C ABI with host buffers: H2D poses from pinned
    # memory, the step, D2H wrenches and taxel maps, every step
    hx = torch.tensor(s.xpos, dtype=torch.float64).pin_memory().numpy()
    hm = torch.tensor(s.xmat, dtype=torch.float64).pin_memory().numpy()
    hv = torch.tensor(s.vel, dtype=torch.float64).pin_memory().numpy()
    h2d = hx.nbytes + hm.nbytes + hv.nbytes
    d2h = n_pair * 6 * 8 + len(s.sensors) * 256 * 4
    e2e_ms = []
    for _ in range(max(3, args.steps // 2)):
        with torch.cuda.stream(stream):
            flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eng.set_poses(hx, hm, hv)
        eng.step()
        w = eng.wrenches()
        tx = eng.all_taxels()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e = n_pair * world / (statistics.median(e2e_ms) * 1e-3)
    launches = eng.launch_count()

    narrow_avg = sum(narrow_ms) / len(narrow_ms)
    achieved = narrow_bytes / (narrow_avg * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (fp64 section values and wrench sums)", "data": "synthetic",
        "config": config_dict(args, world, {"pairs": n_pair, "polygons": n_poly, "tets_touched": n_tets,
                                            "tris_touched": n_tris, "adjoint": "not built"}),
        "e2e": {"value": e2e, "unit": "pairs/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches * args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": None, "kernel": "narrow_kernel",
                     "kernel_ms": narrow_avg, "algorithmic_bytes": narrow_bytes,
                     "step_algorithmic_bytes": step_bytes},
        "clocks": clk,
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.cpu_sample, rank)
    eng.close()
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    import oracle
    n = args.cpu_sample
    s = workload(n, 0)
    o = oracle.Oracle(s)
    for _ in range(args.warmup):
        o.collide()
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        o.collide()
        ts.append(time.perf_counter() - t0)
    o.close()
    t = sum(ts) / len(ts)
    v = n / t
    line = {"metric": METRIC, "value": v, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": config_dict(args, world, {"scenes_per_step": n}),
            "cpu_baseline": {"value": v, "unit": "pairs/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": f"{n} scenes of the workload per step (FP64 oracle, OpenMP over pairs)"},
            "e2e": {"value": v, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
