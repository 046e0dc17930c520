"""Case description: the reference's case-file inputs, parsed and validated.

MicroFC cases are Python scripts that print a JSON dictionary whose keys are
the Fortran namelist names (``'m'``, ``'bc_x%beg'``, ``'patch_icpp(2)%vel(1)'``,
``'fluid_pp(1)%gamma'`` ...; see examples/*/case.py and
toolchain/mfc/run/case_dicts.py of the reference).  ``Case.from_dict`` accepts
exactly that dictionary, so an existing case file drives this library
unchanged; ``Case.to_namelist`` writes the ``&user_inputs`` namelist the
reference's simulation reads (src/simulation/m_start_up.fpp:73-95).
"""
from __future__ import annotations

import dataclasses
import re
from dataclasses import dataclass, field

MAX_FLUIDS = 4
DFLT_INT = -100          # m_global_parameters.fpp:38
DFLT_REAL = -1e6         # m_global_parameters.fpp:37


@dataclass
class Patch:
    """One initial-condition patch (pre_process patch_icpp)."""
    geometry: int                       # 1 line, 2 circle, 3 rectangle, 4 sweep line, 5 ellipse,
                                        # 6 isentropic vortex, 7 2-D analytical, 8 sphere, 9 cuboid,
                                        # 15 1-D analytical, 18 varcircle
    centroid: tuple = (0.0, 0.0, 0.0)
    length: tuple = (0.0, 0.0, 0.0)
    radius: float = 0.0
    smoothen: bool = False
    smooth_patch_id: int = 0            # 0 -> the patch itself (reference default)
    smooth_coeff: float = 0.0
    alter_patch: tuple = ()             # ids of earlier patches this one may overwrite (0 is implied)
    alpha_rho: tuple = ()
    alpha: tuple = ()
    vel: tuple = (0.0, 0.0, 0.0)
    pres: float = 0.0
    normal: tuple = (0.0, 0.0, 0.0)     # sweep line: normal of the line, pointing into the patch
    radii: tuple = (0.0, 0.0, 0.0)      # ellipse: semi-axes along x and y
    epsilon: float = 0.0                # varcircle: thickness of the annulus


def stretch_map(x: float, a: float, lo: float, hi: float) -> float:
    """The hyperbolic stretching factor of a grid coordinate
    (m_grid.f90:79-83), as the input check evaluates it on the domain's ends
    (m_start_up.fpp:261-276)."""
    import math
    return (a + math.log(math.cosh(a * (x - lo))) + math.log(math.cosh(a * (x - hi)))
            - 2.0 * math.log(math.cosh(0.5 * a * (hi - lo)))) / a


@dataclass
class Case:
    m: int
    n: int = 0
    p: int = 0
    x_domain: tuple = (0.0, 1.0)
    y_domain: tuple = (0.0, 0.0)
    z_domain: tuple = (0.0, 0.0)
    dt: float = 0.0
    t_step_start: int = 0
    t_step_stop: int = 1
    t_step_save: int = 1
    num_fluids: int = 1
    time_stepper: int = 3
    weno_order: int = 5
    weno_eps: float = 1e-16
    bc_x: tuple = (-3, -3)
    bc_y: tuple = (DFLT_INT, DFLT_INT)
    bc_z: tuple = (DFLT_INT, DFLT_INT)
    gammas: tuple = ()                  # fluid_pp(i)%gamma  = 1/(gamma_i - 1)
    pi_infs: tuple = ()                 # fluid_pp(i)%pi_inf = gamma_i*pi_inf_i/(gamma_i - 1)
    re_shear: tuple = ()                # fluid_pp(i)%Re(1), shear Reynolds number (<= 0 or absent: inviscid)
    re_bulk: tuple = ()                 # fluid_pp(i)%Re(2), bulk Reynolds number
    # weno_Re_flux: the viscous stresses from WENO-reconstructed velocity
    # gradients (m_viscous.fpp:200-216, m_rhs.fpp:514-528) instead of the
    # finite differences of the default; WENO5, 1-D and 2-D
    weno_re_flux: bool = False
    patches: list = field(default_factory=list)
    stretch_x: tuple = ()               # (a_x, x_a, x_b, loops_x) of a stretched x grid; () = uniform
    stretch_y: tuple = ()               # (a_y, y_a, y_b, loops_y)
    precision: str = "fp64"             # "fp64", "split", "gated" (split + learned WENO gate) or
                                        # "fp64_fma" (FP64 with multiply-add contraction, 2-D WENO5)
    # WENO of the characteristic fields instead of the primitive variables
    # (case key "char_decomp"; no counterpart in the reference, which
    # reconstructs primitive variables): FP64, 1-D to 3-D, WENO3/5
    char_decomp: bool = False
    name: str = "case"

    # index layout, m_global_parameters.fpp:302-310
    @property
    def viscous(self) -> bool:
        return any(r > 0 for r in tuple(self.re_shear) + tuple(self.re_bulk))

    @property
    def num_dims(self) -> int:
        return 1 + min(1, self.n) + min(1, self.p)

    @property
    def sys_size(self) -> int:
        return 2 * self.num_fluids + self.num_dims + 1

    @property
    def mom_idx(self) -> int:
        return self.num_fluids

    @property
    def E_idx(self) -> int:
        return self.num_fluids + self.num_dims

    @property
    def adv_idx(self) -> int:
        return self.num_fluids + self.num_dims + 1

    @property
    def buff_size(self) -> int:
        return (self.weno_order - 1) // 2 + 2

    @property
    def cells(self) -> int:
        return (self.m + 1) * (self.n + 1) * (self.p + 1)

    @property
    def shape(self) -> tuple:
        """Shape of a state array: [S, p+1, n+1, m+1] (x fastest)."""
        return (self.sys_size, self.p + 1, self.n + 1, self.m + 1)

    def replace(self, **kw) -> "Case":
        return dataclasses.replace(self, **kw)

    # -- validation, after s_check_input_file (m_start_up.fpp:117-290) ------
    def check(self) -> None:
        def bad(msg):
            raise ValueError(msg + ". Exiting ...")
        if self.m <= 0:
            bad("Unsupported value of m")
        if self.n < 0 or self.p < 0:
            bad("Unsupported value of n")
        if self.dt <= 0:
            bad("Unsupported value of dt")
        if self.t_step_start < 0:
            bad("Unsupported value of t_step_start")
        if self.t_step_stop <= self.t_step_start:
            bad("Unsupported combination of values of t_step_start and t_step_stop")
        if self.t_step_save > self.t_step_stop - self.t_step_start:
            bad("Unsupported combination of values of t_step_start, t_step_stop and t_step_save")
        if not 1 <= self.num_fluids <= MAX_FLUIDS:
            bad("Unsupported value of num_fluids")
        if self.weno_order not in (1, 3, 5):
            bad("Unsupported value of weno_order")
        if self.m + 1 < 5 * self.weno_order:
            bad("Unsupported combination of values of m and weno_order")
        if self.n + 1 < min(1, self.n) * 5 * self.weno_order:
            bad("Unsupported combination of values of n and weno_order")
        if not (0.0 < self.weno_eps <= 1e-6):
            bad("Unsupported value of weno_eps")
        if self.time_stepper not in (1, 2, 3):
            bad("Unsupported value of time_stepper")
        for name, bc, used in (("bc_x", self.bc_x, True), ("bc_y", self.bc_y, self.n > 0),
                               ("bc_z", self.bc_z, self.p > 0)):
            if not used:
                if tuple(bc) != (DFLT_INT, DFLT_INT):
                    bad(f"Unsupported combination of values of n and {name}%beg")
                continue
            for v in bc:
                if v < -12 or v > -1:
                    bad(f"Unsupported value of {name}%beg")
            if (bc[0] == -1) != (bc[1] == -1):
                bad(f"Unsupported combination of values of {name}%beg and {name}%end")
        if len(self.gammas) < self.num_fluids or len(self.pi_infs) < self.num_fluids:
            bad("Unsupported value of fluid_pp(i)%gamma")
        for g, pi in zip(self.gammas[: self.num_fluids], self.pi_infs[: self.num_fluids]):
            if g <= 0:
                bad("Unsupported value of fluid_pp(i)%gamma")
            if pi < 0:
                bad("Unsupported value of fluid_pp(i)%pi_inf")
        if self.precision not in ("fp64", "split", "gated", "fp64_fma"):
            bad("Unsupported value of precision mode")
        if self.char_decomp and (self.precision != "fp64" or self.viscous or self.weno_order == 1):
            bad("char_decomp needs plain FP64, an inviscid case and WENO3 or WENO5")
        if self.weno_re_flux and self.viscous and (self.precision == "fp64_fma" or self.weno_order != 5):
            bad("weno_Re_flux = T (WENO-reconstructed velocity gradients for the viscous stresses) is built "
                "for WENO5 in the FP64, split and gated precisions")
        # grid stretching, m_start_up.fpp:238-330 (pre_process)
        for ax, st, dom, used in (("x", self.stretch_x, self.x_domain, True),
                                  ("y", self.stretch_y, self.y_domain, self.n > 0)):
            if not st:
                continue
            if not used:
                bad(f"Unsupported choice of the combination of values for n and stretch_{ax}")
            a, lo, hi, loops = st
            for name, v in ((f"a_{ax}", a), (f"{ax}_a", lo), (f"{ax}_b", hi)):
                if v == DFLT_REAL:
                    bad(f"Unsupported choice of the combination of values for stretch_{ax} and {name}")
            if lo >= hi:
                bad(f"Unsupported choice of the combination of values for stretch_{ax}, {ax}_a and {ax}_b")
            for end, v in (("beg", dom[0]), ("end", dom[1])):
                if stretch_map(v, a, lo, hi) <= 0.0:
                    bad(f"Unsupported choice of the combination of values for {ax}_domain%{end}, "
                        f"stretch_{ax}, a_{ax}, {ax}_a, and {ax}_b")
            if loops < 1:
                bad(f"Unsupported choice for the value of loops_{ax}")

    # -- case-file dictionary --------------------------------------------------
    @classmethod
    def from_dict(cls, d: dict) -> "Case":
        """Build a case from a reference case-file dictionary."""
        def num(v):
            if isinstance(v, str):
                s = v.strip().strip("'\"")
                if s.upper() in ("T", ".TRUE."):
                    return True
                if s.upper() in ("F", ".FALSE."):
                    return False
                try:
                    return float(s) if any(c in s for c in ".eE") else int(s)
                except ValueError:
                    return s
            return v

        g = {k: num(v) for k, v in d.items()}
        nf = int(g.get("num_fluids", 1))
        gam = [0.0] * nf
        pinf = [0.0] * nf
        res = [[0.0] * nf, [0.0] * nf]
        patches: dict[int, dict] = {}
        rx = re.compile(r"patch_icpp\((\d+)\)%(\w+)(?:\((\d+)\))?")
        rf = re.compile(r"fluid_pp\((\d+)\)%(\w+)")
        rre = re.compile(r"fluid_pp\((\d+)\)%Re\(([12])\)")
        for k, v in g.items():
            mr = rre.fullmatch(k)
            if mr:
                i = int(mr.group(1)) - 1
                if i < nf:
                    res[int(mr.group(2)) - 1][i] = float(v)
                continue
            mf = rf.fullmatch(k)
            if mf:
                i = int(mf.group(1)) - 1
                if i < nf:
                    if mf.group(2) == "gamma":
                        gam[i] = float(v)
                    elif mf.group(2) == "pi_inf":
                        pinf[i] = float(v)
                continue
            mp = rx.fullmatch(k)
            if mp:
                pid, key, sub = int(mp.group(1)), mp.group(2), mp.group(3)
                pd = patches.setdefault(pid, {})
                if sub is not None:
                    pd.setdefault(key, {})[int(sub)] = v
                else:
                    pd[key] = v
        n = int(g.get("n", 0))
        p = int(g.get("p", 0))
        nd = 1 + min(1, n) + min(1, p)
        plist = []
        for pid in sorted(patches):
            pd = patches[pid]
            vecs = lambda key, cnt, dflt=0.0: tuple(float(pd.get(key, {}).get(i + 1, dflt)) for i in range(cnt))
            alter = tuple(sorted(k for k, v in pd.get("alter_patch", {}).items() if v is True or v == 1))
            plist.append(Patch(
                geometry=int(pd.get("geometry", 0)),
                centroid=(float(pd.get("x_centroid", 0.0)), float(pd.get("y_centroid", 0.0)),
                          float(pd.get("z_centroid", 0.0))),
                length=(float(pd.get("length_x", 0.0)), float(pd.get("length_y", 0.0)),
                        float(pd.get("length_z", 0.0))),
                radius=float(pd.get("radius", 0.0)),
                smoothen=bool(pd.get("smoothen", False)),
                smooth_patch_id=int(pd.get("smooth_patch_id", 0)),
                smooth_coeff=float(pd.get("smooth_coeff", 0.0)),
                alter_patch=alter,
                alpha_rho=vecs("alpha_rho", nf), alpha=vecs("alpha", nf),
                vel=vecs("vel", 3)[:3] if nd else (0.0,), pres=float(pd.get("pres", 0.0)),
                normal=vecs("normal", 3), radii=vecs("radii", 3), epsilon=float(pd.get("epsilon", 0.0))))
        bcy = (int(g.get("bc_y%beg", DFLT_INT)), int(g.get("bc_y%end", DFLT_INT)))
        stretch = {}
        for ax in ("x", "y"):
            if g.get(f"stretch_{ax}", False) in (True, 1):
                stretch[ax] = (float(g.get(f"a_{ax}", DFLT_REAL)), float(g.get(f"{ax}_a", DFLT_REAL)),
                               float(g.get(f"{ax}_b", DFLT_REAL)), int(g.get(f"loops_{ax}", 1)))
        bcz = (int(g.get("bc_z%beg", DFLT_INT)), int(g.get("bc_z%end", DFLT_INT)))
        return cls(
            m=int(g["m"]), n=n, p=p,
            x_domain=(float(g.get("x_domain%beg", 0.0)), float(g.get("x_domain%end", 1.0))),
            y_domain=(float(g.get("y_domain%beg", 0.0)), float(g.get("y_domain%end", 0.0))),
            z_domain=(float(g.get("z_domain%beg", 0.0)), float(g.get("z_domain%end", 0.0))),
            dt=float(g.get("dt", 0.0)),
            t_step_start=int(g.get("t_step_start", 0)), t_step_stop=int(g.get("t_step_stop", 1)),
            t_step_save=int(g.get("t_step_save", 1)),
            num_fluids=nf, time_stepper=int(g.get("time_stepper", 3)),
            weno_order=int(g.get("weno_order", 5)), weno_eps=float(g.get("weno_eps", 1e-16)),
            bc_x=(int(g.get("bc_x%beg", -3)), int(g.get("bc_x%end", -3))), bc_y=bcy, bc_z=bcz,
            gammas=tuple(gam), pi_infs=tuple(pinf), re_shear=tuple(res[0]), re_bulk=tuple(res[1]), patches=plist,
            stretch_x=stretch.get("x", ()), stretch_y=stretch.get("y", ()),
            precision=str(g.get("gpu_precision", "fp64")), name=str(g.get("case_name", "case")),
            char_decomp=str(g.get("char_decomp", "F")).strip().upper() in ("T", "TRUE", ".TRUE.", "1"),
            weno_re_flux=g.get("weno_Re_flux", False) in (True, 1))

    def to_namelist(self) -> str:
        """The &user_inputs namelist of the reference's simulation.inp."""
        L = ["&user_inputs", "case_dir = '.'", "run_time_info = F",
             f"m = {self.m}", f"n = {self.n}", f"dt = {self.dt!r}",
             f"t_step_start = {self.t_step_start}", f"t_step_stop = {self.t_step_stop}",
             f"t_step_save = {self.t_step_save}", f"num_fluids = {self.num_fluids}",
             f"time_stepper = {self.time_stepper}", f"weno_order = {self.weno_order}",
             f"weno_eps = {self.weno_eps!r}", f"bc_x%beg = {self.bc_x[0]}", f"bc_x%end = {self.bc_x[1]}"]
        if self.n > 0:
            L += [f"bc_y%beg = {self.bc_y[0]}", f"bc_y%end = {self.bc_y[1]}"]
        for i in range(self.num_fluids):
            L += [f"fluid_pp({i + 1})%gamma = {self.gammas[i]!r}", f"fluid_pp({i + 1})%pi_inf = {self.pi_infs[i]!r}"]
        L += ["parallel_io = F", "/"]
        return "\n".join(L) + "\n"
