"""Grid and initial condition: the reference's pre_process, vectorised.

* grid: uniform, src/pre_process/m_grid.f90:54-70, or stretched by the
  hyperbolic map of m_grid.f90:72-90
* patches, src/pre_process/m_create_patches.fpp:47-534: line segment (1),
  circle (2), rectangle (3), sweep line (4), ellipse (5), isentropic vortex
  (6), 2-D analytical (7), 1-D analytical (15) and varcircle (18); sphere (8)
  and cuboid (9) are the 3-D analogues of 2 and 3 (the reference's patches
  are 1-D and 2-D; its 2-D ones are z-independent here in 3-D)
* smoothed-patch blending: src/pre_process/m_assign_patches.fpp:54-165
* prim -> cons: src/common/m_variables_conversion.fpp:385-443

Returns the cell boundaries x_cb(-1:m), y_cb(-1:n), z_cb(-1:p) and the
conservative state [S, p+1, n+1, m+1] that the simulation reads from
p_all/p0/0/*.dat.
"""
from __future__ import annotations

import numpy as np

from .case import Case


def uniform_grid(m: int, beg: float, end: float):
    dx = (end - beg) / float(m + 1)
    i = np.arange(m + 1, dtype=np.float64)
    cc = beg + 5e-1 * dx * (2.0 * i + 1.0)
    cb = np.empty(m + 2)
    cb[:-1] = beg + dx * i
    cb[-1] = end
    return cb, cc, dx


_GEOMETRIES_1D = (1, 15)
_GEOMETRIES_2D = (2, 3, 4, 5, 6, 7, 18)
_GEOMETRIES_3D = (8, 9)


def check_patches(case: Case) -> None:
    """Refuses what the device generator refuses: a geometry the grid's
    dimensionality does not take (the line segments are x-slabs in any
    dimension; 2-D patches need n > 0, spheres and cuboids p > 0), a
    smooth_patch_id outside the patches on a patch that blends, an ellipse
    with a non-positive semi-axis and a sweep line with a zero normal."""
    nd, P = case.num_dims, len(case.patches)
    for ip, pt in enumerate(case.patches):
        g = pt.geometry
        ok = g in _GEOMETRIES_1D or (g in _GEOMETRIES_2D and nd >= 2) or (g in _GEOMETRIES_3D and nd == 3)
        if not ok:
            raise ValueError(f"patch {ip + 1}: unsupported patch geometry {g} for a {nd}-D grid")
        sid = pt.smooth_patch_id if pt.smooth_patch_id else ip + 1
        if g in (2, 4, 5, 8) and not 1 <= sid <= P:
            raise ValueError(f"patch {ip + 1}: smooth_patch_id out of range")
        if g == 5 and not (pt.radii[0] > 0 and pt.radii[1] > 0):
            raise ValueError(f"patch {ip + 1}: ellipse semi-axes must be positive")
        if g == 4 and pt.normal[0] == 0 and pt.normal[1] == 0:
            raise ValueError(f"patch {ip + 1}: sweep line normal is zero")


def stretched_grid(cb: np.ndarray, a: float, lo: float, hi: float, loops: int):
    """Stretches uniform cell boundaries x_cb(-1:m) as pre_process does
    (m_grid.f90:72-90): coordinates scaled by the domain length, the
    hyperbolic map applied `loops` times, then scaled back; the centres are
    the boundaries' midpoints and the spacing the smallest width."""
    length = abs(cb[-1] - cb[0])
    cb = cb / length
    lo = lo / length
    hi = hi / length
    for _ in range(loops):
        cb = cb / a * (a + np.log(np.cosh(a * (cb - lo))) + np.log(np.cosh(a * (cb - hi)))
                       - 2.0 * np.log(np.cosh(a * (hi - lo) / 2.0)))
    cb = cb * length
    cc = (cb[1:] + cb[:-1]) / 2.0
    return cb, cc, float(np.min(cb[1:] - cb[:-1]))


def case_grid_1d(m: int, domain, stretch=()):
    """(x_cb, x_cc, dx) of one direction: uniform, then stretched if asked."""
    cb, cc, d = uniform_grid(m, *domain)
    if stretch:
        cb, cc, d = stretched_grid(cb, *stretch)
    return cb, cc, d


def generate(case: Case):
    """Initial condition of a case; returns (x_cb, y_cb, z_cb, q_cons)."""
    m, n, p = case.m, case.n, case.p
    nf, nd, S = case.num_fluids, case.num_dims, case.sys_size
    mb, E, ab = case.mom_idx, case.E_idx, case.adv_idx
    x_cb, xcc, dx = case_grid_1d(m, case.x_domain, case.stretch_x)
    y_cb, ycc, dy = case_grid_1d(n, case.y_domain, case.stretch_y) if n > 0 else (None, np.zeros(1), 0.0)
    z_cb, zcc, dz = uniform_grid(p, *case.z_domain) if p > 0 else (None, np.zeros(1), 0.0)
    Z, Y, X = np.meshgrid(zcc, ycc, xcc, indexing="ij")
    shape = (p + 1, n + 1, m + 1)
    prim = np.zeros((S,) + shape)
    pid = np.zeros(shape, dtype=np.int64)

    check_patches(case)
    for ip, pt in enumerate(case.patches):
        alter = np.isin(pid, (0,) + tuple(pt.alter_patch))
        eta = np.ones(shape)
        xc, yc, zc = pt.centroid
        lx, ly, lz = pt.length
        g = pt.geometry
        smooth_id = pt.smooth_patch_id if pt.smooth_patch_id else ip + 1
        if g in (1, 15):
            hit = ((xc - 0.5 * lx) <= X) & ((xc + 0.5 * lx) >= X) & alter
        elif g in (3, 7, 9):
            hit = (((xc - 0.5 * lx) <= X) & ((xc + 0.5 * lx) >= X) &
                   ((yc - 0.5 * ly) <= Y) & ((yc + 0.5 * ly) >= Y) & alter)
            if g == 9:
                hit &= ((zc - 0.5 * lz) <= Z) & ((zc + 0.5 * lz) >= Z)
        elif g in (2, 8):
            r2 = (X - xc) * (X - xc) + (Y - yc) * (Y - yc)
            h = min(dx, dy)
            if g == 8:
                r2 = r2 + (Z - zc) * (Z - zc)
                h = min(h, dz)
            if pt.smoothen:
                eta = np.tanh(pt.smooth_coeff / h * (np.sqrt(r2) - pt.radius)) * (-0.5) + 0.5
            hit = ((r2 <= pt.radius * pt.radius) & alter) | (pid == smooth_id)
        elif g == 4:  # s_sweep_line, m_create_patches.fpp:323-371
            a, b = pt.normal[0], pt.normal[1]
            c = -a * xc - b * yc
            lin = a * X + b * Y + c
            if pt.smoothen:
                eta = 5e-1 + 5e-1 * np.tanh(pt.smooth_coeff / min(dx, dy) * lin / np.sqrt(a * a + b * b))
            hit = ((lin >= 0.0) & alter) | (pid == smooth_id)
        elif g == 5:  # s_ellipse, m_create_patches.fpp:202-250
            u = (X - xc) / pt.radii[0]
            v = (Y - yc) / pt.radii[1]
            r2 = u * u + v * v
            if pt.smoothen:
                eta = np.tanh(pt.smooth_coeff / min(dx, dy) * (np.sqrt(r2) - 1.0)) * (-0.5) + 0.5
            hit = ((r2 <= 1.0) & alter) | (pid == smooth_id)
        elif g == 6:  # s_isentropic_vortex, m_create_patches.fpp:379-419
            hit = ((X - xc) * (X - xc) + (Y - yc) * (Y - yc) <= pt.radius * pt.radius) & alter
        elif g == 18:  # s_varcircle, m_create_patches.fpp:151-194
            r = np.sqrt((X - xc) * (X - xc) + (Y - yc) * (Y - yc))
            hit = (r <= pt.radius + pt.epsilon / 2.0) & (r >= pt.radius - pt.epsilon / 2.0) & alter
        else:
            raise ValueError(f"unsupported patch geometry {g}")
        if not hit.any():
            continue
        e = eta[hit]
        orig = prim[:, hit].copy()
        for f in range(nf):
            prim[f][hit] = e * pt.alpha_rho[f] + (1.0 - e) * orig[f]
            prim[ab + f][hit] = e * pt.alpha[f] + (1.0 - e) * orig[ab + f]
        for d in range(nd):
            prim[mb + d][hit] = e * pt.vel[d] + (1.0 - e) * orig[mb + d]
        prim[E][hit] = e * pt.pres + (1.0 - e) * orig[E]
        if g in (7, 15):
            # pressure bump about the centroid at the cells' right boundaries
            # x_cb(i), y_cb(j) (m_create_patches.fpp:462-464, 523-525)
            XB = np.broadcast_to(x_cb[1:].reshape(1, 1, -1), shape)
            s2 = (XB - xc) * (XB - xc)
            if g == 7:
                YB = np.broadcast_to(y_cb[1:].reshape(1, -1, 1), shape)
                s2 = s2 + (YB - yc) * (YB - yc)
            prim[E][hit] = prim[E][hit] * (1.0 + 0.2 * np.exp(-1.0 * s2[hit] / (2.0 * 0.005)))
        owner = pid[hit]
        owner[(1.0 - e) < 1e-16] = ip + 1
        pid[hit] = owner

    # prim -> cons, m_variables_conversion.fpp:406-443
    q = np.empty_like(prim)
    rho = np.zeros(shape)
    gam = np.zeros(shape)
    pinf = np.zeros(shape)
    for f in range(nf):
        rho = rho + prim[f]
        gam = gam + prim[ab + f] * case.gammas[f]
        pinf = pinf + prim[ab + f] * case.pi_infs[f]
    q[:nf] = prim[:nf]
    dyn = np.zeros(shape)
    for d in range(nd):
        q[mb + d] = rho * prim[mb + d]
        dyn = dyn + q[mb + d] * prim[mb + d] / 2.0
    q[E] = gam * prim[E] + dyn + pinf
    q[ab:ab + nf] = prim[ab:ab + nf]
    return x_cb, y_cb, z_cb, q


def grid(case: Case):
    """The cell boundaries x_cb, y_cb, z_cb of a case (None when unused)."""
    x_cb = case_grid_1d(case.m, case.x_domain, case.stretch_x)[0]
    y_cb = case_grid_1d(case.n, case.y_domain, case.stretch_y)[0] if case.n > 0 else None
    z_cb = uniform_grid(case.p, *case.z_domain)[0] if case.p > 0 else None
    return x_cb, y_cb, z_cb


def device_patches(case: Case):
    """(mfc_patch array, domain[6]) of a case for the device generator
    (mfc_gpu_generate_ic); the same patch semantics as generate().  The
    domain is None on a stretched grid: the generator then takes the
    context's cell boundaries."""
    from . import _lib
    P = len(case.patches)
    if not 1 <= P <= _lib.MFC_MAX_PATCHES:
        raise ValueError(f"{P} patches; the device generator takes 1..{_lib.MFC_MAX_PATCHES}")
    arr = (_lib.MfcPatch * P)()
    for i, pt in enumerate(case.patches):
        a = arr[i]
        a.geometry = pt.geometry
        a.x_centroid, a.y_centroid, a.z_centroid = pt.centroid
        a.length_x, a.length_y, a.length_z = pt.length
        a.radius = pt.radius
        a.smoothen = int(pt.smoothen)
        a.smooth_patch_id = pt.smooth_patch_id if pt.smooth_patch_id else i + 1
        a.smooth_coeff = pt.smooth_coeff
        for j in range(_lib.MFC_MAX_PATCHES + 1):
            a.alter_patch[j] = 1 if (j == 0 or j in pt.alter_patch) else 0
        for f in range(case.num_fluids):
            a.alpha_rho[f] = pt.alpha_rho[f]
            a.alpha[f] = pt.alpha[f]
        for d in range(3):
            a.vel[d] = pt.vel[d] if d < len(pt.vel) else 0.0
            a.normal[d] = pt.normal[d] if d < len(pt.normal) else 0.0
            a.radii[d] = pt.radii[d] if d < len(pt.radii) else 0.0
        a.pres = pt.pres
        a.epsilon = pt.epsilon
    if case.stretch_x or case.stretch_y:
        return arr, None
    dom = np.array([*case.x_domain, *case.y_domain, *case.z_domain], dtype=np.float64)
    return arr, dom


def to_primitive(case: Case, q: np.ndarray) -> np.ndarray:
    """cons -> prim (m_variables_conversion.fpp:326-373) of a whole state, FP64."""
    nf, nd = case.num_fluids, case.num_dims
    mb, E, ab = case.mom_idx, case.E_idx, case.adv_idx
    prim = q.copy()
    rho = np.zeros(q.shape[1:])
    gam = np.zeros(q.shape[1:])
    pinf = np.zeros(q.shape[1:])
    for f in range(nf):
        rho = rho + q[f]
        gam = gam + q[ab + f] * case.gammas[f]
        pinf = pinf + q[ab + f] * case.pi_infs[f]
    rho = np.maximum(rho, 1e-16)
    dyn = np.zeros(q.shape[1:])
    for d in range(nd):
        prim[mb + d] = q[mb + d] / rho
        dyn = dyn + 0.5 * q[mb + d] * prim[mb + d]
    prim[E] = (q[E] - dyn - pinf) / gam
    return prim


def max_wave_dt(case: Case, q: np.ndarray, cfl: float, x_cb, y_cb=None, z_cb=None) -> float:
    """dt = cfl * min over cells of min_d dx_d/(|u_d| + c), with the mixture
    sound speed of the reference's ICFL monitor (m_data_output.fpp:215-221)."""
    prim = to_primitive(case, q)
    nf, nd = case.num_fluids, case.num_dims
    mb, E, ab = case.mom_idx, case.E_idx, case.adv_idx
    rho = sum(prim[f] for f in range(nf))
    gam = sum(prim[ab + f] * case.gammas[f] for f in range(nf))
    pinf = sum(prim[ab + f] * case.pi_infs[f] for f in range(nf))
    c = np.sqrt(((gam + 1.0) * prim[E] + pinf) / (gam * rho))
    cbs = (x_cb, y_cb, z_cb)
    best = np.inf
    for d in range(nd):
        w = np.diff(np.asarray(cbs[d]))
        shp = [1, 1, 1]
        shp[2 - d] = -1
        best = min(best, float(np.min(w.reshape(shp) / (np.abs(prim[mb + d]) + c))))
    return cfl * best
