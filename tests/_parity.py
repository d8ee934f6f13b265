"""Comparison helpers shared by the parity tests."""
from __future__ import annotations

import numpy as np

# Tolerances (FP32 GPU vs FP64 oracle).
WRENCH_RTOL = 1e-5     # force: |dF| <= 1e-5 |F|; torque (about M's origin, as
                       # reported): |dT| <= 1e-5 (|T| + |F| (sqrt(area) + arm)),
                       # arm = distance from M's origin to the contact centroid
AREA_RTOL = 1e-5
TAXEL_RTOL = 1e-5      # relative to the largest taxel of the map


def compare_candidates(gpu: np.ndarray, orc: np.ndarray):
    """Candidate sets and polygon vertex counts after a canonical sort.

    Rows are (pair, elem_a, elem_b, n_vert, flags); flag bit 0 marks a
    near-degenerate element pair (a value within 1e-12 of a clip plane).
    Returns (mismatches, n_near, n_common) where mismatches lists keys that
    differ and are not near-degenerate on the side(s) that have them.
    """
    g = {(int(r[0]), int(r[1]), int(r[2])): (int(r[3]), int(r[4])) for r in gpu}
    o = {(int(r[0]), int(r[1]), int(r[2])): (int(r[3]), int(r[4])) for r in orc}
    bad, near = [], 0
    for k in sorted(set(g) | set(o)):
        gi, oi = g.get(k), o.get(k)
        flagged = bool((gi and gi[1] & 1) or (oi and oi[1] & 1))
        near += flagged
        if gi and oi:
            if gi[0] != oi[0] and not flagged:
                bad.append((k, gi, oi))
        elif not flagged:
            bad.append((k, gi, oi))
    return bad, near, len(set(g) & set(o))


def wrench_errors(wg: np.ndarray, wo: np.ndarray, area: np.ndarray, centroid=None, xm=None):
    """Relative force and torque errors per pair.  The torque is the reported
    one (about M's origin); its scale is |T| + |F| (sqrt(area) + arm), the
    force times the lever arm from M's origin to the oracle's contact centroid
    plus the contact's size, so that neither a torque that nearly vanishes
    about M's origin (a force through it) nor one about a far origin sets a
    scale the force's own rounding does not have."""
    Fg, Fo, Tg, To = wg[:, :3], wo[:, :3], wg[:, 3:], wo[:, 3:]
    fo = np.linalg.norm(Fo, axis=1)
    arm = np.zeros(len(fo)) if centroid is None or xm is None else np.linalg.norm(
        np.asarray(centroid) - np.asarray(xm), axis=1)
    ef = np.linalg.norm(Fg - Fo, axis=1) / np.maximum(fo, 1e-9)
    et = np.linalg.norm(Tg - To, axis=1) / np.maximum(np.linalg.norm(To, axis=1) + fo * (np.sqrt(area) + arm),
                                                      1e-12)
    return ef, et


def taxel_check(tg: np.ndarray, to: np.ndarray, sample_bound: float):
    """Taxel maps agree within TAXEL_RTOL of the map maximum, except cells
    whose difference is at most one ray sample (a sample within float rounding
    of a contact-triangle edge can be missed or hit twice by either ray
    caster, as in the reference's own).  Returns (n_bad, n_sample_cells)."""
    scale = max(float(np.abs(to).max()), 1e-12)
    d = np.abs(tg.astype(np.float64) - to.astype(np.float64))
    ok = d <= TAXEL_RTOL * scale
    one_sample = (~ok) & (d <= sample_bound * 1.001 + TAXEL_RTOL * scale)
    bad = int(np.sum(~ok & ~one_sample))
    return bad, int(np.sum(one_sample))
