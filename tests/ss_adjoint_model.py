"""FP64 numpy model of the soft-soft contact polygons of one pair and of the
hand-written reverse of their wrench (test infrastructure, CPU).

It restates, in FP64 and per element pair, what the device computes:
  * the polygon: tet A's section by p_A(x) = p_B(x), clipped by tet B's four
    faces (Drake's ComputeContactSurfaceFromCompliantVolumes, called at
    mujoco_contact_surfaces_plugin.cpp:284-286), with the two constraint
    labels of every vertex (0-3: A's face opposite vertex k, 4 + j: B's face
    opposite vertex j), as the device's tet_section / clip_dist record them;
  * the kTriangle / kPolygon quadrature and the force law
    (mujoco_contact_surfaces_plugin.cpp:320-409, 435-483), soft frame = A's;
  * the reverse of both and the contraction with the vertex tangents under a
    twist (w, v) of body B in A's frame, line by line as the device's
    wrench_adjoint_ss (adjoint.cuh), with the determinant guard as a
    parameter so that an FP32 evaluation can be emulated.
The tests compare the model's forward with the oracle and its reverse with
central differences of the model itself.
"""
from __future__ import annotations

import numpy as np

COS_ALPHA = -0.38268343236508978   # cos(5 pi / 8)
NEAR = 1e-12
EPS_SLIP = (1e-4 * 1e-2) ** 2


def tet_field(X, P):
    g = np.linalg.solve(X[1:] - X[0], P[1:] - P[0])
    return g, P[0] - g @ X[0]


def face_normals(X):
    """Unnormalised normals of the faces opposite vertex 0..3."""
    out = []
    for k in range(4):
        o = [i for i in range(4) if i != k]
        out.append(np.cross(X[o[1]] - X[o[0]], X[o[2]] - X[o[0]]))
    return out


def tet_planes(X):
    """Inward unit normals and offsets of the faces opposite vertex 0..3."""
    pn, po = [], []
    for k, nrm in enumerate(face_normals(X)):
        o = [i for i in range(4) if i != k]
        nrm = nrm / np.linalg.norm(nrm)
        if nrm @ (X[k] - X[o[0]]) < 0:
            nrm = -nrm
        pn.append(nrm)
        po.append(nrm @ X[o[0]])
    return pn, po


def tet_section(X, s):
    pos = [s[k] > 0 for k in range(4)]
    npos = sum(pos)
    if npos in (0, 4):
        return [], False
    near = any(abs(x) < NEAR for x in s)
    if npos in (1, 3):
        single = pos.index(True) if npos == 1 else pos.index(False)
        edges = [(single, k) for k in range(4) if k != single]
    else:
        a, b = [k for k in range(4) if pos[k]]
        c, d = [k for k in range(4) if not pos[k]]
        edges = [(a, c), (a, d), (b, d), (b, c)]
    out = []
    for a, b in edges:
        lab = tuple(k for k in range(4) if k not in (a, b))
        if abs(s[a]) > abs(s[b]):
            a, b = b, a
        t = s[a] / (s[a] - s[b])
        out.append((X[a] + t * (X[b] - X[a]), lab))
    return out, near


def orient_ccw(poly, up):
    """The finished polygon wound counter-clockwise about up (the direction in
    which the section value grows), first vertex kept: the device's polygons
    wind that way (it winds the section before clipping, which keeps the
    winding, so its first vertex may differ; the reverse does not depend on
    it)."""
    x = [v for v, _ in poly]
    w = sum(np.cross(x[i - 1] - x[0], x[i] - x[0]) @ up for i in range(2, len(x)))
    return [poly[0]] + poly[1:][::-1] if w < 0 else poly


def _shared(la, lb):
    return la[0] if la[0] in lb else la[1]


def clip(poly, pn, po, j):
    d = [pn @ x - po for x, _ in poly]
    near = any(abs(v) < NEAR for v in d)
    if all(v >= 0 for v in d):
        return poly, near
    out = []
    n = len(poly)
    for i in range(n):
        k = (i + 1) % n
        di, dk = d[i], d[k]
        if di >= 0:
            out.append(poly[i])
        if (di >= 0) != (dk >= 0):
            if abs(di) <= abs(dk):
                x = poly[i][0] + di / (di - dk) * (poly[k][0] - poly[i][0])
            else:
                x = poly[k][0] + dk / (dk - di) * (poly[i][0] - poly[k][0])
            out.append((x, (_shared(poly[i][1], poly[k][1]), 4 + j)))
    return out, near


def element_polygon(XA, PA, XB, PB):
    """The polygon of one element pair (A's frame), or None."""
    gA, cA = tet_field(XA, PA)
    gB, cB = tet_field(XB, PB)
    m = gA - gB
    lm = np.linalg.norm(m)
    n = m / lm
    if not (n @ gA / np.linalg.norm(gA) > COS_ALPHA and -(n @ gB) / np.linalg.norm(gB) > COS_ALPHA):
        return None
    s = [(PA[k] - (gB @ XA[k] + cB)) / lm for k in range(4)]
    poly, near = tet_section(XA, s)
    if not poly:
        return None
    pn, po = tet_planes(XB)
    for j in range(4):
        poly, nj = clip(poly, pn[j], po[j], j)
        near = near or nj
        if len(poly) < 3:
            return None
    poly = orient_ccw(poly, n)
    return dict(x=[x for x, _ in poly], lab=[lab for _, lab in poly], n=n, gA=gA, cA=cA, gB=gB, lm=lm,
                gM=gA @ n, gN=-(gB @ n), faceA=face_normals(XA), pnB=pn, near=near)


def _point_force(F, T, A, p, n, gM, gN, p0, vf):
    lin, ang, damping, mu = vf
    if not A > 1e-14 or gM < 1e-14 or gN < 1e-14:
        return
    g = 1.0 / (1.0 / gM + 1.0 / gN)
    v = lin + np.cross(ang, p)
    vn = v @ n
    fn = max(0.0, 1.0 - damping * vn) * (A * p0 - 0.001 * A * g * vn)
    vt = v - n * vn
    vs = np.sqrt(vt @ vt + EPS_SLIP)
    s = vs / 1e-4
    mur = mu * s * (2 - s) if s < 1 else mu
    f = (n - mur * vt / vs) * fn
    F += f
    T += np.cross(p, f)


def _fan(x, pr, n):
    A, c, pc = 0.0, np.zeros(3), 0.0
    for i in range(1, len(x) - 1):
        ai = 0.5 * np.cross(x[i] - x[0], x[i + 1] - x[0]) @ n
        A += ai
        c = c + ai * (x[0] + x[i] + x[i + 1]) / 3
        pc += ai * (pr[0] + pr[i] + pr[i + 1]) / 3
    return A, c, pc


def polygon_wrench(P, vf, repr_=0):
    """Force and torque about A's origin (A's frame) of one polygon."""
    x, n = P['x'], P['n']
    pr = [P['gA'] @ xi + P['cA'] for xi in x]
    A, c, pc = _fan(x, pr, n)
    F, T = np.zeros(3), np.zeros(3)
    if A == 0:
        return F, T
    c, pc = c / A, pc / A
    if repr_ == 1:
        _point_force(F, T, abs(A), c, n, P['gM'], P['gN'], pc, vf)
        return F, T
    for i in range(len(x)):
        j = (i + 1) % len(x)
        Ai = 0.5 * np.linalg.norm(np.cross(x[i] - c, x[j] - c))
        _point_force(F, T, Ai, (c + x[i] + x[j]) / 3, n, P['gM'], P['gN'], pc / 3 + pr[i] / 3 + pr[j] / 3, vf)
    return F, T


def _point_reverse(gF, gT, A, p, n, gM, gN, p0, vf):
    lin, ang, damping, mu = vf
    if not A > 1e-14 or gM < 1e-14 or gN < 1e-14:
        return None
    g = 1.0 / (1.0 / gM + 1.0 / gN)
    fn0, k = A * p0, A * g
    v = lin + np.cross(ang, p)
    vn = v @ n
    h = 1.0 - damping * vn
    hp = max(0.0, h)
    fnb = fn0 - 0.001 * k * vn
    fn = hp * fnb
    vt = v - n * vn
    vs = np.sqrt(vt @ vt + EPS_SLIP)
    s = vs / 1e-4
    mur = mu * s * (2 - s) if s < 1 else mu
    u = vt / vs
    q = n - u * mur
    f = q * fn
    fbar = gF + np.cross(gT, p)
    Lfn = fbar @ q
    qbar = fbar * fn
    nbar = qbar.copy()
    murbar = -(qbar @ u)
    ubar = qbar * (-mur)
    vtbar = ubar / vs
    vsbar = -(ubar @ vt) / (vs * vs) + murbar * (mu * (2 - 2 * s) / 1e-4 if s < 1 else 0.0)
    vtbar = vtbar + vt * (vsbar / vs)
    vbar = vtbar.copy()
    vnbar = -(vtbar @ n)
    nbar = nbar - vtbar * vn
    hbar = Lfn * fnb if h > 0 else 0.0
    fn0bar = Lfn * hp
    kbar = -Lfn * hp * 0.001 * vn
    vnbar += -Lfn * hp * 0.001 * k - damping * hbar
    vbar = vbar + n * vnbar
    nbar = nbar + v * vnbar
    gbar = kbar * A
    return dict(A=kbar * g + fn0bar * p0, p0=fn0bar * A, gM=gbar * (g / gM) ** 2, gN=gbar * (g / gN) ** 2,
                p=np.cross(vbar, ang) + np.cross(f, gT), n=nbar, d=-hbar * vn)


def polygon_reverse(P, gF, gT, vf, repr_=0, anc=None, det_tol=1e-12, moduli=None):
    """dL/d(w, v) of one polygon for L = gF . F + gT . T (the device's
    wrench_adjoint_ss).  With `anc`, the vertices are relative to it (the
    device keeps them so in FP32); det_tol: the dependent-rows guard.  With
    moduli = (E_A, E_B), returns (dL/d(w, v), dL/dE_A, dL/dE_B, dL/d(damping))
    instead, the moduli's own terms at fixed damping."""
    x, n = list(P['x']), P['n']
    anc = np.zeros(3) if anc is None else anc
    ga, gb, lm = P['gA'], P['gB'], P['lm']
    pv = [ga @ xi + P['cA'] for xi in x]
    nv = len(x)
    xb = [np.zeros(3) for _ in range(nv)]
    pb = [0.0] * nv
    A, Sc, Sp = _fan(x, pv, n)
    if A == 0:
        return np.zeros(6)
    iA = 1.0 / A
    c, pc = Sc * iA, Sp * iA
    nbar, cbar = np.zeros(3), np.zeros(3)
    gMbar = gNbar = pcbar = Abar = gD = 0.0
    if repr_ == 1:
        b = _point_reverse(gF, gT, abs(A), anc + c, n, P['gM'], P['gN'], pc, vf)
        if b is not None:
            Abar += -b['A'] if A < 0 else b['A']
            cbar = cbar + b['p']
            pcbar += b['p0']
            nbar = nbar + b['n']
            gMbar += b['gM']
            gNbar += b['gN']
            gD += b['d']
    for i in range(nv if repr_ == 0 else 0):
        j = (i + 1) % nv
        u, w = x[i] - c, x[j] - c
        cr = np.cross(u, w)
        ln = np.linalg.norm(cr)
        b = _point_reverse(gF, gT, 0.5 * ln, anc + (c + x[i] + x[j]) / 3, n, P['gM'], P['gN'],
                           pc / 3 + pv[i] / 3 + pv[j] / 3, vf)
        if b is None:
            continue
        nbar = nbar + b['n']
        gMbar += b['gM']
        gNbar += b['gN']
        gD += b['d']
        if ln > 0:
            crb = cr * (0.5 * b['A'] / ln)
            ub, wb = np.cross(w, crb), np.cross(crb, u)
            xb[i] = xb[i] + ub
            xb[j] = xb[j] + wb
            cbar = cbar - ub - wb
        c3 = b['p'] / 3
        cbar = cbar + c3
        xb[i] = xb[i] + c3
        xb[j] = xb[j] + c3
        pcbar += b['p0'] / 3
        pb[i] += b['p0'] / 3
        pb[j] += b['p0'] / 3
    Scb, Spb = cbar * iA, pcbar * iA
    Abar -= (cbar @ c + pcbar * pc) * iA
    for i in range(1, nv - 1):
        e1, e2 = x[i] - x[0], x[i + 1] - x[0]
        cr = np.cross(e1, e2)
        ai = 0.5 * cr @ n
        aib = Abar + Scb @ (x[0] + x[i] + x[i + 1]) / 3 + Spb * (pv[0] + pv[i] + pv[i + 1]) / 3
        sx, sp = Scb * (ai / 3), Spb * ai / 3
        for q in (0, i, i + 1):
            xb[q] = xb[q] + sx
            pb[q] += sp
        nbar = nbar + cr * (0.5 * aib)
        e1b, e2b = np.cross(e2, n) * (0.5 * aib), np.cross(n, e1) * (0.5 * aib)
        xb[i] = xb[i] + e1b
        xb[i + 1] = xb[i + 1] + e2b
        xb[0] = xb[0] - e1b - e2b
    nbar = nbar + ga * gMbar - gb * gNbar
    npp = nbar - n * (nbar @ n)
    rot = np.cross(npp, gb) / lm + np.cross(n, gb) * gNbar
    tr = np.zeros(3)
    iEa, iEb = (1.0 / moduli[0], 1.0 / moduli[1]) if moduli is not None else (0.0, 0.0)
    gEa = (npp @ ga / lm + gMbar * P['gM']) * iEa
    gEb = (gNbar * P['gN'] - npp @ gb / lm) * iEb
    for v in range(nv):
        xe = xb[v] + ga * pb[v]
        gEa += pb[v] * pv[v] * iEa
        l0, l1 = P['lab'][v]
        r1 = P['faceA'][l0] if l0 < 4 else P['pnB'][l0 - 4]
        r2 = P['faceA'][l1] if l1 < 4 else P['pnB'][l1 - 4]
        a0, a1, a2 = np.cross(r1, r2), np.cross(r2, n), np.cross(n, r1)
        det = n @ a0
        if not abs(det) > det_tol * np.linalg.norm(n) * np.linalg.norm(r1) * np.linalg.norm(r2):
            # dependent rows: the vertex lies on the line r1 = r2 = 0, which
            # the section contains (both pressures vanish there); the two
            # face rows alone carry its motion (minimum norm: no slide along
            # the line)
            g11, g12, g22 = r1 @ r1, r1 @ r2, r2 @ r2
            gd = g11 * g22 - g12 * g12
            if not gd > det_tol * g11 * g22:
                continue
            q1, q2 = r1 @ xe, r2 @ xe
            B = np.zeros(3)
            if l0 >= 4:
                B = B + r1 * ((g22 * q1 - g12 * q2) / gd)
            if l1 >= 4:
                B = B + r2 * ((g11 * q2 - g12 * q1) / gd)
            tr = tr + B
            rot = rot + np.cross(anc + x[v], B)
            continue
        b0 = xe @ a0 / det
        B = gb * (-b0 / lm)
        if l0 >= 4:
            B = B + r1 * (xe @ a1 / det)
        if l1 >= 4:
            B = B + r2 * (xe @ a2 / det)
        tr = tr + B
        rot = rot + np.cross(anc + x[v], B)
        gEa -= b0 * pv[v] / lm * iEa
        gEb += b0 * pv[v] / lm * iEb
    if moduli is not None:
        return np.concatenate([rot, tr]), gEa, gEb, gD
    return np.concatenate([rot, tr])


def as_float32(P):
    """The polygon as the device holds it: vertices relative to the first one
    (a point of tet A's neighbourhood, as the device's anchor vertex) and every
    operand rounded to FP32.  Returns (polygon, anchor)."""
    anc = np.asarray(P['x'][0], np.float64)
    Q = dict(P)
    Q['x'] = [np.float32(xi - anc) for xi in P['x']]
    for k in ('n', 'gA', 'gB'):
        Q[k] = np.float32(P[k])
    Q['cA'] = np.float32(P['cA'] + P['gA'] @ anc)
    Q['lm'] = np.float32(P['lm'])
    Q['gM'] = np.float32(P['gM'])
    Q['gN'] = np.float32(P['gN'])
    Q['faceA'] = [np.float32(f) for f in P['faceA']]
    Q['pnB'] = [np.float32(f) for f in P['pnB']]
    return Q, np.float32(anc)
