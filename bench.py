"""Benchmark of the batched hydroelastic contact step (forward + adjoint) on GB300.

python bench.py --gpus N --steps K --warmup W [--impl reference]

Workload: 4096 independent tactile scenes per GPU (rigid 8x8 cm plate with a
16x16 taxel grid, 5x5 rays per cell, pressed by a soft sphere / ellipsoid /
cylinder of 2k-8k tets, E in 5e4-5e5 Pa, penetration 0-4 mm, in-plane offset
+-2 cm, velocities U[-0.1,0.1]): the differentiable batched workload.  One
step = pair frames, LBVH broadphase, clipping, quadrature, Hunt-Crossley +
friction, per-pair wrenches, taxel binning, then the adjoint of the wrenches
and taxel maps with respect to both bodies' poses and the modulus (seeded
upstream gradients).  Synthetic seeded inputs: no dataset exists.

`value` is timed with inputs resident in HBM, each step one CUDA graph of
the forward step and its adjoint (hc_step_adjoint_device); `e2e` goes through
the C ABI with host buffers (hc_step_adjoint: poses and upstream gradients in,
wrenches, taxel maps and gradients out every step, one wait).  The plain path (one scene per launch sequence,
no graph) is timed on a sample for the batched/plain ratio.  `--impl
reference` times the CPU path (the FP64 restatement in oracle/, OpenMP over
pairs, all host threads) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "contact pairs/s fwd+adjoint, batched vs plain GPU path at 1e-5 rel wrench err"

# DRAM bytes of one narrow_sr_keep_kernel launch (dram__bytes_read.sum +
# dram__bytes_write.sum) from an ncu capture of this workload at 1024 scenes
# (launch shape 6,2), scaled by the scenes processed (items and polygons
# grow in proportion).
NARROW_SR_DRAM_BYTES_PER_SCENE = (61.00736e6 + 30.865664e6) / 1024


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--scenes", type=int, default=4096)
    ap.add_argument("--cpu-sample", type=int, default=256, help="scenes in the CPU baseline sample")
    ap.add_argument("--plain-sample", type=int, default=64, help="scenes timed on the plain path")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--launch-shape", default=None,
                    help="CTAS,CHUNK: use this launch shape instead of autotuning (e.g. the shape an earlier "
                         "run chose, for a profiler run whose own timings would mislead the autotuner)")
    ap.add_argument("--taxel-sensors", type=int, default=0,
                    help="K: also attach a taxel-point sensor with a KxK taxel grid to every plate")
    return ap.parse_args()


def dist_info():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(
        os.environ.get("LOCAL_RANK", "0"))


def max_over_ranks(x: float, world: int) -> float:
    """The largest per-rank value (the slowest rank's step time); a gloo
    all-reduce on the host, no device collective."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t[0])


def workload(n_scenes, rank):
    """The tactile scenes; the plate is 0.1 mm wider in x than in y so that no
    ray sample lies exactly on its top face's diagonal (where any two ray
    casters may disagree by one sample)."""
    from mujoco_contact_surfaces_gb300 import scenes
    return scenes.tactile(n_scenes, seed=scenes.SEED_ADJOINT + rank, velocities=True,
                          plate_half=(0.0401, 0.04, 0.005))


def sample_pairs(n_pair, n_sample):
    """Evenly spaced pairs of the workload: the CPU legs' bounded sample."""
    n = min(n_sample, n_pair)
    return sorted({int(round(k * (n_pair - 1) / max(1, n - 1))) for k in range(n)})


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


def upstream(s, seed=17):
    """Seeded dL/dwrench (n_pair x 6) and dL/dtaxel (all maps)."""
    rng = np.random.default_rng(seed)
    return rng.normal(size=(len(s.g1), 6)), rng.normal(size=256 * len(s.sensors)).astype(np.float32) * 1e-3


def config_dict(args, world, extra=None):
    c = {"workload": f"tactile batched fwd+adjoint: {args.scenes} scenes/GPU, rigid 8x8 cm plate + 16x16 taxels "
                     "(5x5 rays/cell) vs soft sphere/ellipsoid/cylinder 2k-8k tets",
         "scenes_per_gpu": args.scenes, "pairs_per_scene": 1, "representation": "kTriangle",
         "l2": "flushed between timed steps (256 MiB write)", "parallelism": f"scene shards x{world}"}
    if extra:
        c.update(extra)
    return c


def cpu_sample_scene(s, n_sample):
    from mujoco_contact_surfaces_gb300 import scenes
    pairs = sample_pairs(len(s.g1), n_sample)
    return pairs, scenes.subscene(s, pairs)


def cpu_baseline(sub, n_pairs, reps=3):
    """FP64 oracle, OpenMP over pairs, all host cores, on a bounded sample of
    the workload's pairs (forward only: the reference path has no adjoint)."""
    import oracle
    o = oracle.Oracle(sub)
    o.collide()
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        o.collide()
        ts.append(time.perf_counter() - t0)
    o.close()
    t = statistics.median(ts)
    return {"value": n_pairs / t, "unit": "pairs/s", "cores": os.cpu_count(), "cpu_model": cpu_model(),
            "kind": "port",
            "sample": f"{n_pairs} evenly spaced scenes of the timed workload (one pair and one 16x16 sensor each), "
                      f"forward only (the reference path has no adjoint), FP64, OpenMP over pairs, median of {reps}"}


def accuracy(sub, pairs, w, stats, taxels):
    """The timed step's wrenches, contact areas and taxel maps of the sampled
    pairs against the FP64 oracle on the same pairs (outside the timed
    region).  Taxel errors are relative to each map's largest value."""
    import oracle
    o = oracle.Oracle(sub)
    ref = o.collide()
    o.close()
    F, Fo = w[pairs, :3], ref["wrench"][:, :3]
    T, To = w[pairs, 3:], ref["wrench"][:, 3:]
    fo = np.linalg.norm(Fo, axis=1)
    area_ref = ref["area"]
    # torque scale: |T| + |F| (sqrt(area) + lever arm from M's origin to the
    # oracle's contact centroid)
    arm = np.linalg.norm(ref["centroid"] - ref["xm"], axis=1)
    ef = np.linalg.norm(F - Fo, axis=1) / np.maximum(fo, 1e-9)
    et = np.linalg.norm(T - To, axis=1) / np.maximum(np.linalg.norm(To, axis=1) + fo * (np.sqrt(area_ref) + arm),
                                                     1e-12)
    area = np.array([stats[p].area for p in pairs])
    nz = area_ref > 0
    ea = np.abs(area[nz] - area_ref[nz]) / area_ref[nz]
    # a cell may differ by one ray sample (a ray within float rounding of a
    # contact-polygon edge is hit or missed by either caster); one sample
    # weighs p / 25 and is bounded by twice the map's largest value / 25
    t_err, t_all, one = 0.0, 0.0, 0
    one_sample = 2.0 / 25.0 * 1.001 + 1e-5
    for j, p in enumerate(pairs):
        to = ref["taxels"][j].astype(np.float64)
        scale = max(float(np.abs(to).max()), 1e-12)
        d = np.abs(taxels[p].astype(np.float64) - to) / scale
        sample_off = (d > 1e-5) & (d <= one_sample)
        one += int(np.sum(sample_off))
        t_err = max(t_err, float(d[~sample_off].max(initial=0.0)))
        t_all = max(t_all, float(d.max()))
    return {"n_pairs": len(pairs), "n_touching": int(np.sum(nz)), "max_rel_wrench_err": float(max(ef.max(), et.max())),
            "max_rel_force_err": float(ef.max()), "max_rel_torque_err": float(et.max()),
            "max_rel_area_err": float(ea.max(initial=0.0)), "max_taxel_err_frac": t_err,
            "taxel_cells_one_ray_sample_off": one, "max_taxel_err_frac_incl_those": t_all,
            "taxel_cells": 256 * len(pairs),
            "oracle": "FP64 CPU restatement (oracle/), same pairs, same poses"}


class Clocks:
    def __init__(self, device):
        self.device = device
        self.proc = None
        # the raw samples (the JSON line carries their summary): HC_CLOCKS_DIR
        # or the system's temporary directory
        out_dir = os.environ.get("HC_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(out_dir, f"clocks_{os.getpid()}.csv")

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
    """Bytes per step by the per-pair formula: forward 80 B per distinct soft
    tet and 48 B per distinct rigid triangle with a non-empty polygon, 96 B of
    poses, 48 B of wrench, 1024 B of taxels per sensor pair; the adjoint reads
    the same elements again plus 48 B of dL/dwrench and 1024 B of dL/dtaxel
    and writes 104 B of gradients."""
    eng.set_debug(1)
    eng.step()
    cand = eng.candidates()
    eng.set_debug(0)
    tets = len(np.unique(cand[:, 0] * (1 << 32) + cand[:, 1]))
    rig = cand[cand[:, 2] >= 0]
    tris = len(np.unique(rig[:, 0] * (1 << 32) + rig[:, 2]))
    elem = 80 * tets + 48 * tris
    fwd = elem + (96 + 48) * n_pair + 1024 * n_sensor_pairs
    adj = fwd + (48 + 104) * n_pair + 1024 * n_sensor_pairs
    return dict(elem=elem, fwd=fwd, adj=adj, step=fwd + adj, tets=tets, tris=tris, polygons=len(cand))


def plain_path(s_full, n_sample, dLdw, dLdt, local):
    """One scene per launch sequence, no graph: its own context per scene,
    fwd + adjoint, timed sequentially."""
    import torch
    from mujoco_contact_surfaces_gb300 import scenes
    sub = scenes.Scene()
    # the first n_sample scenes (pair k = scene k, geoms 2k, 2k+1)
    engines = []
    for k in range(n_sample):
        sc = scenes.Scene()
        for g in (s_full.geoms[2 * k], s_full.geoms[2 * k + 1]):
            sc.add_geom(g["type"], g["size"], g["cs5"], g["mesh_v"], g["mesh_f"])
        sc.xpos = s_full.xpos[2 * k:2 * k + 2].copy()
        sc.xmat = s_full.xmat[2 * k:2 * k + 2].copy()
        sc.vel = s_full.vel[2 * k:2 * k + 2].copy()
        sc.g1, sc.g2 = [0], [1]
        sn = dict(s_full.sensors[k])
        sn["geom"] = 1
        sc.sensors = [sn]
        e = scenes.build_engine(sc, device=local, use_graph=False)
        e.set_adjoint_mode(True)
        engines.append((e, sc, dLdw[k:k + 1], dLdt[256 * k:256 * (k + 1)]))
    del sub
    for e, sc, dw, dt in engines[:2]:
        e.step()
        e.wrenches()
        e.adjoint(dw, dt)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for e, sc, dw, dt in engines:
        e.set_poses(sc.xpos, sc.xmat, sc.vel)
        e.step()
        e.wrenches()
        e.taxels(0)
        e.adjoint(dw, dt)
    t = time.perf_counter() - t0
    launches = engines[0][0].launch_count() + engines[0][0].adjoint_launch_count()
    for e, *_ in engines:
        e.close()
    return n_sample / t, launches


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
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"

    s = workload(args.scenes, rank)
    n_pair = len(s.g1)
    eng = scenes.build_engine(s, device=local)
    extra = {}
    if args.taxel_sensors > 0:
        from mujoco_contact_surfaces_gb300 import _lib as L
        k = args.taxel_sensors
        g = np.linspace(-0.035, 0.035, k)
        grid = np.array([[x, y, 0.005] for x in g for y in g])
        for sn in s.sensors:
            eng.add_taxel_sensor(sn["geom"], grid, L.TAXEL_SQUARED, 0.002, 0.0015, L.SAMPLE_DEFAULT, False)
        eng.set_pairs(s.g1, s.g2)
        extra["taxel_sensors"] = {"per_plate": k * k, "method": "squared", "include_margin": 0.002,
                                  "sample_resolution": 0.0015, "sample_method": "default"}
    eng.set_adjoint_mode(True)
    if args.launch_shape:
        tuned_ctas, tuned_chunk = (int(x) for x in args.launch_shape.split(","))
        eng.set_launch_shape(tuned_ctas, tuned_chunk)
    else:
        tuned_ctas, tuned_chunk = eng.autotune()   # launch shape, before any timing
    eng.enable_timing(True)
    ab = algorithmic_bytes(eng, n_pair, len(s.sensors))
    dLdw_h, dLdt_h = upstream(s)

    stream = torch.cuda.ExternalStream(eng.stream(), device=local)
    dev = torch.device("cuda", local)
    xpos = torch.tensor(s.xpos, dtype=torch.float64, device=dev)
    xmat = torch.tensor(s.xmat, dtype=torch.float64, device=dev)
    vel = torch.tensor(s.vel, dtype=torch.float64, device=dev)
    dLdw = torch.tensor(dLdw_h, dtype=torch.float64, device=dev)
    dLdt = torch.tensor(dLdt_h, dtype=torch.float32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    n_geom = s.n_geom
    torch.cuda.synchronize()

    def device_step():
        # forward step and adjoint: one graph launch
        eng.set_poses_device(n_geom, xpos.data_ptr(), xmat.data_ptr(), vel.data_ptr())
        eng.step_adjoint_device(dLdw.data_ptr(), dLdt.data_ptr())

    for _ in range(args.warmup):
        device_step()
    eng.wrenches()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()

    clocks = Clocks(local)
    clocks.start()
    step_ms, narrow_ms, kept_ms, adj_ms = [], [], [], []
    e0, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(2))
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1)
            e0.record(stream)
        device_step()
        with torch.cuda.stream(stream):
            e2.record(stream)
        e2.synchronize()
        step_ms.append(e0.elapsed_time(e2))
        tm = eng.timings()   # the engine's stage events inside the graph
        adj_ms.append(tm.ms_adjoint)
        narrow_ms.append(tm.ms_narrowphase)
        kept_ms.append(tm.ms_kept_polygons)
    torch.cuda.synchronize()
    clk = clocks.stop()
    t_step = max_over_ranks(sum(step_ms) / len(step_ms), world)
    value = n_pair * world / (t_step * 1e-3)
    launches = eng.launch_count() + eng.adjoint_launch_count()

    # end to end through the C ABI with host buffers every step
    hx = torch.tensor(s.xpos, dtype=torch.float64).pin_memory().numpy()
    hm = torch.tensor(s.xmat, dtype=torch.float64).pin_memory().numpy()
    hv = torch.tensor(s.vel, dtype=torch.float64).pin_memory().numpy()
    hw = torch.tensor(dLdw_h, dtype=torch.float64).pin_memory().numpy()
    ht = torch.tensor(dLdt_h, dtype=torch.float32).pin_memory().numpy()
    h2d = hx.nbytes + hm.nbytes + hv.nbytes + hw.nbytes + ht.nbytes
    d2h = n_pair * 6 * 8 + len(s.sensors) * 256 * 4 + n_pair * 14 * 8
    d2h += len(s.sensors) * args.taxel_sensors ** 2 * 4
    # results land in page-locked host arrays the caller owns (direct copies)
    pinned = lambda shape, dt: torch.zeros(shape, dtype=dt).pin_memory().numpy()
    ow = pinned((n_pair, 6), torch.float64)
    otx = pinned((len(s.sensors) * 256,), torch.float32)
    ots = pinned((len(s.sensors) * args.taxel_sensors ** 2,), torch.float32)
    odp = pinned((n_pair, 2, 6), torch.float64)
    odE = pinned((n_pair, 2), torch.float64)
    e2e_ms = []
    for _ in range(max(3, args.steps // 2)):
        with torch.cuda.stream(stream):
            flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        # poses and upstream gradients in, wrenches, taxel maps and gradients
        # out: one call, one wait (hc_step_adjoint)
        eng.step_adjoint(hx, hm, hv, hw, ht, out=(ow, otx, odp, odE))
        if args.taxel_sensors > 0:
            eng.all_taxel_sensor_values(out=ots)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e = n_pair * world / (max_over_ranks(statistics.median(e2e_ms), world) * 1e-3)

    narrow_avg = sum(narrow_ms) / len(narrow_ms)
    kept_avg = sum(kept_ms) / len(kept_ms)
    adj_avg = sum(adj_ms) / len(adj_ms)
    # roofline of the kernel that reads the algorithmic element bytes (the
    # soft-rigid narrow phase; the kept-polygon passes read records, which
    # are overhead by the formula)
    kname, kms, kbytes = "narrow_sr_keep_kernel", narrow_avg, ab["elem"]
    achieved = kbytes / (kms * 1e-3) / 1e9
    traffic = NARROW_SR_DRAM_BYTES_PER_SCENE * args.scenes
    line = {
        "metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (fp64 section values, plane offsets and wrench sums)",
        "data": "synthetic (seeded PCG64 scenes; no dataset exists)",
        "config": config_dict(args, world, {"pairs": n_pair, "polygons": ab["polygons"],
                                            # secondary figure: non-empty element pairs (polygons)
                                            # through forward and adjoint, per second, all ranks
                                            "element_pairs_per_s": ab["polygons"] * world / (t_step * 1e-3),
                                            "tets_touched": ab["tets"],
                                            "tris_touched": ab["tris"], "ms_forward": t_step - adj_avg,
                                            # forward alone (like for like with the CPU legs)
                                            "forward_pairs_per_s": n_pair * world / ((t_step - adj_avg) * 1e-3),
                                            "ms_adjoint": adj_avg, "ms_narrow_kernel": narrow_avg,
                                            "ms_kept_polygons_pass": kept_avg,
                                            "autotuned": {"ctas_per_sm": tuned_ctas, "chunk": tuned_chunk},
                                            **extra}),
        "e2e": {"value": e2e, "unit": "pairs/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches * args.steps,
        "launches_per_step": launches, "graphs_per_step": 1,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": traffic,
                     "traffic_source": "ncu dram bytes of one launch at 1024 scenes, scaled by scenes",
                     "kernel": kname, "kernel_ms": kms,
                     "algorithmic_bytes": kbytes,
                     # the whole step by the per-pair formula: B_fwd + B_adj, the
                     # adjoint reading the elements again
                     "step_algorithmic_bytes": ab["step"],
                     "step_achieved_gbs": ab["step"] / (t_step * 1e-3) / 1e9,
                     "step_frac": ab["step"] / (t_step * 1e-3) / 1e9 / hbm_peak, "peak_source": peak_src},
        "clocks": clk,
    }
    # accuracy of the timed step on a sample of its pairs (outside the timed
    # region): the last step's outputs against the FP64 oracle
    w_last = eng.wrenches()
    stats = eng.pair_stats()
    tax = eng.all_taxels().reshape(len(s.sensors), -1)
    pairs, sub = cpu_sample_scene(s, args.cpu_sample)
    line["accuracy"] = accuracy(sub, pairs, w_last, stats, tax)
    eng.close()
    if rank == 0 and not args.no_plain:
        pv, pl = plain_path(s, min(args.plain_sample, len(s.g1)), dLdw_h, dLdt_h, local)
        line["config"]["plain_pairs_per_s"] = pv
        # device-timed batched over host-timed plain, and host over host
        line["config"]["batched_over_plain"] = value / world / pv
        line["config"]["e2e_over_plain"] = e2e / world / pv
        line["config"]["plain_launches_per_scene"] = pl
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(sub, len(pairs))
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    import oracle
    pairs, s = cpu_sample_scene(workload(args.scenes, 0), args.cpu_sample)
    n = len(pairs)
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
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded PCG64 scenes)", "impl": "reference",
            "config": config_dict(args, world, {"scenes_per_step": n, "pass": "forward only (the reference path "
                                                                            "has no adjoint)"}),
            "cpu_baseline": {"value": v, "unit": "pairs/s", "cores": os.cpu_count(), "cpu_model": cpu_model(),
                             "kind": "port",
                             "sample": f"{n} evenly spaced scenes of the {args.scenes}-scene workload per step "
                                       f"(FP64 oracle, OpenMP over pairs, all host threads)"},
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
