"""The reference's data files: case directory layout and record format.

The simulation reads its initial condition and writes every t_step_save
steps (src/simulation/m_start_up.fpp:298-390, m_data_output.fpp:316-381):

    <case_dir>/p_all/p<rank>/<t_step>/x_cb.dat        x_cb(-1:m)
    <case_dir>/p_all/p<rank>/<t_step>/y_cb.dat        y_cb(-1:n)        (2-D)
    <case_dir>/p_all/p<rank>/<t_step>/q_cons_vf<i>.dat q_cons_vf(i)%sf(0:m,0:n)

and the text files of m_data_output.fpp:387-462 (cons.<i>.<rank>.<t>.dat,
and prim.<i>.<rank>.<t>.dat in 1-D) under <case_dir>/D/.

Each .dat file under p_all is one Fortran unformatted sequential record (gfortran layout): a
4-byte little-endian length marker, the payload, the same marker again.
Records longer than 2**31-9 bytes are split into sub-records whose leading
marker is negated when more sub-records follow (gfortran's scheme).  Arrays
are stored in Fortran (column-major) order, i.e. x fastest, which is also
the x-fastest C order of the [S, p+1, n+1, m+1] state used here.
"""
from __future__ import annotations

import os
import struct

import numpy as np

_MAX_SUB = 2**31 - 9


def write_record(path: str, data: np.ndarray) -> None:
    payload = np.ascontiguousarray(data, dtype="<f8").tobytes()
    with open(path, "wb") as f:
        pos, n = 0, len(payload)
        while True:
            chunk = payload[pos:pos + _MAX_SUB]
            more = pos + len(chunk) < n
            lead = -len(chunk) if more else len(chunk)
            trail = -len(chunk) if pos > 0 else len(chunk)
            f.write(struct.pack("<i", lead))
            f.write(chunk)
            f.write(struct.pack("<i", trail))
            pos += len(chunk)
            if not more:
                break


def read_record(path: str) -> np.ndarray:
    out = bytearray()
    with open(path, "rb") as f:
        while True:
            hdr = f.read(4)
            if len(hdr) != 4:
                raise ValueError(f"{path}: truncated record marker")
            lead = struct.unpack("<i", hdr)[0]
            size = abs(lead)
            chunk = f.read(size)
            if len(chunk) != size:
                raise ValueError(f"{path}: truncated record ({len(chunk)} of {size} bytes)")
            tail = f.read(4)
            if len(tail) != 4 or abs(struct.unpack("<i", tail)[0]) != size:
                raise ValueError(f"{path}: record markers do not match")
            out += chunk
            if lead >= 0:
                break
    return np.frombuffer(bytes(out), dtype="<f8").copy()


def step_dir(case_dir: str, t_step: int, rank: int = 0) -> str:
    return os.path.join(case_dir, "p_all", f"p{rank}", str(t_step))


def write_data_files(case_dir: str, t_step: int, case, q: np.ndarray, x_cb, y_cb=None, z_cb=None,
                     rank: int = 0) -> str:
    """s_write_serial_data_files: grid and conservative variables of one step."""
    d = step_dir(case_dir, t_step, rank)
    os.makedirs(d, exist_ok=True)
    write_record(os.path.join(d, "x_cb.dat"), np.asarray(x_cb))
    if case.n > 0:
        write_record(os.path.join(d, "y_cb.dat"), np.asarray(y_cb))
    if case.p > 0:
        write_record(os.path.join(d, "z_cb.dat"), np.asarray(z_cb))
    for i in range(case.sys_size):
        write_record(os.path.join(d, f"q_cons_vf{i + 1}.dat"), q[i])
    return d


def read_data_files(case_dir: str, t_step: int, case, rank: int = 0):
    """s_read_serial_data_files: returns (x_cb, y_cb, z_cb, q[S,p+1,n+1,m+1])."""
    d = step_dir(case_dir, t_step, rank)
    if not os.path.isdir(d):
        raise FileNotFoundError(f"{d}/. is missing. Exiting ...")

    def grid(name, count):
        a = read_record(os.path.join(d, name))
        if a.size != count:
            raise ValueError(f"{name}: expected {count} values, found {a.size}")
        return a

    x_cb = grid("x_cb.dat", case.m + 2)
    y_cb = grid("y_cb.dat", case.n + 2) if case.n > 0 else None
    z_cb = grid("z_cb.dat", case.p + 2) if case.p > 0 else None
    q = np.empty(case.shape)
    for i in range(case.sys_size):
        path = os.path.join(d, f"q_cons_vf{i + 1}.dat")
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} is missing. Exiting ...")
        a = read_record(path)
        if a.size != case.cells:
            raise ValueError(f"{path}: expected {case.cells} values, found {a.size}")
        q[i] = a.reshape(case.shape[1:])
    return x_cb, y_cb, z_cb, q


def _fortran_f(x: float, w: int, d: int) -> str:
    """Fortran Fw.d edit of one value (gfortran): right-justified, rounded to
    d decimals, asterisks when it does not fit, NaN/Infinity spelled out."""
    if x != x:
        return "NaN".rjust(w)
    if x in (float("inf"), float("-inf")):
        t = "Infinity" if x > 0 else "-Infinity"
        return t.rjust(w) if len(t) <= w else "*" * w
    t = f"{x:{w}.{d}f}"
    return t if len(t) <= w else "*" * w


def write_text_files(case_dir: str, t_step: int, case, q: np.ndarray, x_cb, y_cb=None, rank: int = 0,
                     precision: int = 2) -> list[str]:
    """The D/ text output of s_write_serial_data_files (m_data_output.fpp:387-462).

    1-D: prim.<i>.<rank>.<t>.dat (partial densities and volume fractions as
    stored, u = rho u / rho, p from the stiffened-gas energy) and
    cons.<i>.<rank>.<t>.dat, one "x_cb(j) value" line per cell.  2-D:
    cons.<i>.<rank>.<t>.dat with "x_cb(j) y_cb(k) value" lines, k fastest,
    and an empty line after each j.  As in the reference, the coordinate
    written for cell j is x_cb(j), the cell's right boundary.  3-D cases get
    no text output (the reference writes none).  precision 1: F30.3 / F30.7,
    otherwise F40.14."""
    out_dir = os.path.join(case_dir, "D")
    os.makedirs(out_dir, exist_ok=True)
    written = []
    xr = np.asarray(x_cb)[1:]  # x_cb(0:m)
    nf = case.num_fluids

    def name(kind, i):
        return os.path.join(out_dir, f"{kind}.{i + 1}.{rank:02d}.{t_step:06d}.dat")

    if case.n == 0:
        w, d = (30, 3) if precision == 1 else (40, 14)
        qq = q.reshape(case.sys_size, -1)
        rho = np.zeros(qq.shape[1])
        gam = np.zeros(qq.shape[1])
        pinf = np.zeros(qq.shape[1])
        for f in range(nf):
            rho = rho + qq[f]
            gam = gam + qq[case.adv_idx + f] * case.gammas[f]
            pinf = pinf + qq[case.adv_idx + f] * case.pi_infs[f]
        for i in range(case.sys_size):
            if i == case.mom_idx:
                val = qq[i] / rho
            elif i == case.E_idx:
                val = (qq[case.E_idx] - 0.5 * (qq[case.mom_idx] ** 2.0) / rho - pinf) / gam
            else:
                val = qq[i]
            path = name("prim", i)
            with open(path, "w") as f:
                f.writelines(_fortran_f(a, w, d) + _fortran_f(b, w, d) + "\n" for a, b in zip(xr, val))
            written.append(path)
        for i in range(case.sys_size):
            path = name("cons", i)
            with open(path, "w") as f:
                f.writelines(_fortran_f(a, w, d) + _fortran_f(b, w, d) + "\n" for a, b in zip(xr, qq[i]))
            written.append(path)
    elif case.p == 0:
        w, d = (30, 7) if precision == 1 else (40, 14)
        yr = [_fortran_f(v, w, d) for v in np.asarray(y_cb)[1:]]
        for i in range(case.sys_size):
            path = name("cons", i)
            field = q[i].reshape(case.n + 1, case.m + 1)
            with open(path, "w") as f:
                for j in range(case.m + 1):
                    xs = _fortran_f(xr[j], w, d)
                    f.writelines(xs + yr[k] + _fortran_f(field[k, j], w, d) + "\n" for k in range(case.n + 1))
                    f.write("\n")
            written.append(path)
    return written
