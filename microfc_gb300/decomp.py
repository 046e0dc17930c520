"""Domain decomposition with halo exchange, on one GPU or across ranks.

``decompose`` splits a case the way s_mpi_decompose_computational_domain
does (src/simulation/m_mpi_proxy.fpp:134-328): (m+1) // p cells per
subdomain, the first (m+1) % p subdomains one more, subdomains ordered x
fastest, then y, then z, a processor boundary (the neighbour's rank, >= 0)
wherever a subdomain meets another one, and the physical boundary
conditions (a periodic one wrapping around to the far subdomain) elsewhere.
The reference decomposes in x and y; z follows the same rule.

Every RK stage needs the neighbours' strips of that stage's input (the
halo exchange of s_populate_conservative_variables_buffers, m_rhs.fpp:434
and m_mpi_proxy.fpp:468-979).  ``MultiDomain`` runs all subdomains on one
GPU: each subdomain packs its strips straight into the neighbours' receive
buffers (mfc_gpu_halo_pack / mfc_gpu_halo_buffer), x strips before y
strips, then every subdomain runs the stage (mfc_gpu_rk_stage).  ``exchange`` is the rank-to-rank form:
send/receive pairs of packed strips through torch.distributed (NCCL between
GPUs, gloo on the host).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .case import Case
from .solver import _dp


@dataclass
class Subdomain:
    rank: int
    coords: tuple            # (ix, iy, iz)
    start: tuple             # first global cell (x, y, z)
    case: Case               # the subdomain's case: local m, n, p and boundary conditions
    x_cb: np.ndarray
    y_cb: np.ndarray | None
    z_cb: np.ndarray | None = None
    neighbors: dict = field(default_factory=dict)  # (dir, side) -> rank

    def window(self):
        """Slices of the global [S, p+1, n+1, m+1] state this subdomain holds."""
        sx, sy, sz = self.start
        c = self.case
        return (slice(None), slice(sz, sz + c.p + 1), slice(sy, sy + c.n + 1), slice(sx, sx + c.m + 1))


def _split(count: int, parts: int):
    base, rem = divmod(count, parts)
    sizes = [base + (1 if i < rem else 0) for i in range(parts)]
    starts = [sum(sizes[:i]) for i in range(parts)]
    return sizes, starts


def decompose(case: Case, x_cb, y_cb=None, px: int = 2, py: int = 1, pz: int = 1, z_cb=None) -> list[Subdomain]:
    """Subdomains of a case on a px x py x pz process grid."""
    if case.n == 0 and py != 1:
        raise ValueError("a 1-D case decomposes along x only")
    if case.p == 0 and pz != 1:
        raise ValueError("a 2-D case does not decompose along z")
    parts = (px, py, pz)
    counts = (case.m + 1, case.n + 1, case.p + 1)
    used = (True, case.n > 0, case.p > 0)
    splits = [_split(counts[d], parts[d]) for d in range(3)]
    for d in range(3):
        if used[d] and min(splits[d][0]) < 5 * case.weno_order:
            raise ValueError("subdomains too small for the WENO stencil")
    cbs = (x_cb, y_cb, z_cb)
    subs = []
    for iz in range(pz):
        for iy in range(py):
            for ix in range(px):
                coords = (ix, iy, iz)
                rank = (iz * py + iy) * px + ix
                bcs = [list(case.bc_x), list(case.bc_y), list(case.bc_z)]
                nb = {}
                for d in range(3):
                    if not used[d]:
                        continue
                    for side in (0, 1):
                        c, n = coords[d], parts[d]
                        inner = (side == 0 and c > 0) or (side == 1 and c < n - 1)
                        if inner or (bcs[d][side] == -1 and n > 1):
                            o = list(coords)
                            o[d] = (c - 1) % n if side == 0 else (c + 1) % n
                            other = (o[2] * py + o[1]) * px + o[0]
                            nb[(d, side)] = other
                            bcs[d][side] = other
                sizes = [splits[d][0][coords[d]] for d in range(3)]
                starts = [splits[d][1][coords[d]] for d in range(3)]
                sub_case = case.replace(m=sizes[0] - 1, n=(sizes[1] - 1) if used[1] else 0,
                                        p=(sizes[2] - 1) if used[2] else 0, bc_x=tuple(bcs[0]), bc_y=tuple(bcs[1]),
                                        bc_z=tuple(bcs[2]), name=f"{case.name}_p{rank}")
                loc = [None if (cbs[d] is None or not used[d]) else
                       np.asarray(cbs[d])[starts[d]:starts[d] + sizes[d] + 1] for d in range(3)]
                subs.append(Subdomain(rank, coords, tuple(starts), sub_case, loc[0], loc[1], loc[2], nb))
    return subs


def _map_x(c: int, n: int, bcb: int, bce: int):
    """Ghost index mapping of one x index (mfc::map_cell): (cell, flip)."""
    if c < 0:
        flip = bcb == -2
        c = c + n if bcb == -1 else (-c - 1 if bcb == -2 else 0)
    elif c >= n:
        flip = bce == -2
        c = c - n if bce == -1 else (2 * n - 1 - c if bce == -2 else n - 1)
    else:
        flip = False
    return min(max(c, 0), n - 1), flip


def halo_strip(sub: Subdomain, q_local: np.ndarray, d: int, side: int, H: int, x_ghosts=None) -> np.ndarray:
    """Host restatement of mfc_gpu_halo_pack: the strip of a local state
    [S, p+1, n+1, m+1] that the neighbour across (d, side) needs, in its
    receive-buffer layout (depth 0 next to the boundary): x [S][p+1][n+1][H],
    y [S][p+1][H][m+1] in 3-D, z [S][H][n+1][m+1].  A 2-D y strip is
    [S][1][H][m+3]: its first and last columns are the x ghost cells -1 and
    m+1 of the packed rows -- x_ghosts = (left, right), each [S, n+1], the
    depth-0 columns this subdomain received across its x processor
    boundaries (None on a side with a physical boundary, which the x
    boundary condition fills)."""
    axis = 3 - d  # array axis of direction d
    n = q_local.shape[axis]
    idx = [k if side == 0 else n - 1 - k for k in range(H)]
    strip = np.take(q_local, idx, axis=axis)  # depth replaces the axis
    c = sub.case
    if d == 1 and c.p == 0:
        m1 = q_local.shape[3]
        cols = []
        for j, x in enumerate((-1, m1)):
            g = None if x_ghosts is None else x_ghosts[j]
            if g is not None:
                col = np.asarray(g)[:, idx]
            else:
                gx, flip = _map_x(x, m1, c.bc_x[0], c.bc_x[1])
                col = q_local[:, 0, idx, gx].copy()
                if flip:
                    col[c.num_fluids] = -col[c.num_fluids]
            cols.append(col[:, None, :, None])
        strip = np.concatenate([cols[0], strip, cols[1]], axis=3)
    return np.ascontiguousarray(strip)


def ghost_widths(neighbor: Subdomain, d: int, side: int, b: int) -> np.ndarray:
    """The b cell widths of `neighbor` next to the boundary it shares with a
    subdomain whose side `side` faces it (depth 0 first): what the reference
    sends in s_mpi_sendrecv_grid_variables_buffers (m_mpi_proxy.fpp:338-458)."""
    w = np.diff(np.asarray((neighbor.x_cb, neighbor.y_cb, neighbor.z_cb)[d]))
    return np.ascontiguousarray(w[::-1][:b] if side == 0 else w[:b])


def exchange(sub: Subdomain, strips: dict, group=None) -> dict:
    """Rank-to-rank halo exchange: sends strips[(d, side)] to the neighbour
    across (d, side) and returns what each neighbour sent, keyed by the side
    it arrives on.  Tensors may live on the host (gloo) or the GPU (NCCL);
    every send is matched by the neighbour's receive on its opposite side, so
    the pattern is the same on every rank and cannot deadlock.  Only the
    sides in `strips` are exchanged: a 2-D run exchanges its x strips first
    and packs its y strips after they arrived (the y strips forward the
    diagonal neighbours' cells), as the reference exchanges x before y."""
    import torch
    import torch.distributed as dist
    reqs, out = [], {}
    for (d, side) in sorted(strips):
        peer = sub.neighbors[(d, side)]
        t = strips[(d, side)]
        buf = torch.empty_like(t)
        out[(d, side)] = buf
        reqs.append(dist.isend(t.contiguous(), dst=peer, group=group, tag=2 * d + side))
        reqs.append(dist.irecv(buf, src=peer, group=group, tag=2 * d + (1 - side)))
    for r in reqs:
        r.wait()
    return out


class MultiDomain:
    """All subdomains of a decomposed case on one GPU, stepped with a halo
    exchange before every RK stage; bit-identical to the undecomposed run."""

    def __init__(self, case: Case, x_cb, y_cb=None, q_cons=None, px: int = 2, py: int = 1, pz: int = 1,
                 z_cb=None, device: int = 0):
        from .solver import Simulation
        self.case = case
        self.subs = decompose(case, x_cb, y_cb, px, py, pz, z_cb)
        self.sims = []
        for s in self.subs:
            q = None if q_cons is None else np.ascontiguousarray(q_cons[s.window()])
            self.sims.append(Simulation(s.case, s.x_cb, s.y_cb, s.z_cb, q_cons=q, device=device, check=False))
        self.L = _lib.load()
        b = (case.weno_order - 1) // 2 + 2  # buff_size
        for s, sim in zip(self.subs, self.sims):
            for (d, side), peer in s.neighbors.items():
                w = ghost_widths(self.subs[peer], d, side, b)
                _lib.check(self.L.mfc_gpu_set_halo_widths(sim._h, d, side, _dp(w), b))

    def close(self):
        for s in self.sims:
            s.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_gate(self, params) -> None:
        """Learned-gate parameters of every subdomain (gated cases)."""
        for sim in self.sims:
            sim.set_gate(params)

    def _buffer(self, rank: int, d: int, side: int) -> int:
        p = ctypes.c_void_p()
        n = ctypes.c_int64()
        _lib.check(self.L.mfc_gpu_halo_buffer(self.sims[rank]._h, d, side, ctypes.byref(p), ctypes.byref(n)))
        return p.value

    def step(self, dt: float) -> None:
        import torch
        nd = 1 + (self.case.n > 0) + (self.case.p > 0)
        for stage in range(self.case.time_stepper):
            # one direction at a time: a 2-D y strip forwards the x ghost
            # cells its subdomain has just received
            for d in range(nd):
                for s, sim in zip(self.subs, self.sims):
                    for (dd, side), peer in s.neighbors.items():
                        if dd != d:
                            continue
                        dst = self._buffer(peer, d, 1 - side)
                        _lib.check(self.L.mfc_gpu_halo_pack(sim._h, stage, d, side, ctypes.c_void_p(dst)))
                torch.cuda.synchronize()
            for sim in self.sims:
                _lib.check(self.L.mfc_gpu_rk_stage(sim._h, stage, float(dt)))
            torch.cuda.synchronize()

    def run(self, t_step_start: int, t_step_stop: int, dt: float | None = None) -> float:
        """The p_main loop (with its last-step dt trim) over the subdomains."""
        dt = self.case.dt if dt is None else dt
        t_step = t_step_start
        mytime = 0.0 if t_step == 0 else t_step * dt
        finaltime = t_step_stop * dt
        while True:
            mytime = mytime + dt
            if t_step == t_step_stop:
                break
            self.step(dt)
            if (mytime + dt) >= finaltime:
                dt = finaltime - mytime
            t_step = t_step + 1
        return dt

    def download(self) -> np.ndarray:
        q = np.empty(self.case.shape)
        for s, sim in zip(self.subs, self.sims):
            q[s.window()] = sim.download()
        return q
