"""The benchmark cases of this project, built as reference-style case inputs.

* ``sod_1d``            1-D two-fluid Sod shock tube (ideal gases, gamma 1.4)
* ``shock_droplet_2d``  2-D air shock (Mach Ms) on a water droplet
* ``shock_bubble_3d``   3-D air shock on a helium sphere (z-extension)

Post-shock states follow the normal-shock (Rankine-Hugoniot) relations of an
ideal gas, as the reference's examples/2D_shockdroplet/case.py states them:
p2/p1 = 1 + 2g/(g+1) (Ms^2 - 1), rho2/rho1 = (g+1) Ms^2 / ((g-1) Ms^2 + 2),
u2 = Ms c1 (1 - rho1/rho2).  dt is set once from the initial state with the
mixture sound speed, dt = cfl * min(dx/(|u|+c)); the reference has no
adaptive dt.
"""
from __future__ import annotations

import math

from .case import Case, Patch
from . import preprocess


def stiffened(gamma: float, pi_inf: float = 0.0):
    """fluid_pp gamma/pi_inf inputs of the reference for a stiffened gas."""
    return 1.0 / (gamma - 1.0), gamma * pi_inf / (gamma - 1.0)


def normal_shock(gamma: float, rho1: float, p1: float, mach: float):
    c1 = math.sqrt(gamma * p1 / rho1)
    p2 = p1 * (1.0 + 2.0 * gamma / (gamma + 1.0) * (mach * mach - 1.0))
    rho2 = rho1 * (gamma + 1.0) * mach * mach / ((gamma - 1.0) * mach * mach + 2.0)
    u2 = mach * c1 * (1.0 - rho1 / rho2)
    return rho2, u2, p2


def sod_1d(m: int = 999, steps: int = 4000, dt: float = 5e-5, eps_alpha: float = 1e-6) -> Case:
    """Two ideal gases (gamma 1.4), [0,1], interface at 0.5; transmissive BCs."""
    g, pi = stiffened(1.4)
    a_hi, a_lo = 1.0 - eps_alpha, eps_alpha
    left = Patch(geometry=1, centroid=(0.25, 0, 0), length=(0.5, 0, 0),
                 alpha_rho=(1.0 * a_hi, 1.0 * a_lo), alpha=(a_hi, a_lo), vel=(0.0, 0, 0), pres=1.0)
    right = Patch(geometry=1, centroid=(0.75, 0, 0), length=(0.5, 0, 0),
                  alpha_rho=(0.125 * a_lo, 0.125 * a_hi), alpha=(a_lo, a_hi), vel=(0.0, 0, 0), pres=0.1)
    return Case(m=m, x_domain=(0.0, 1.0), dt=dt, t_step_stop=steps, t_step_save=steps,
                num_fluids=2, time_stepper=3, weno_order=5, weno_eps=1e-16, bc_x=(-3, -3),
                gammas=(g, g), pi_infs=(pi, pi), patches=[left, right], name=f"sod_1d_{m + 1}")


def shock_droplet_2d(nx: int = 1024, ny: int = 512, mach: float = 1.47, radius: float = 2e-3,
                     steps: int = 1000, cfl: float = 0.3, smooth_coeff: float = 0.5,
                     precision: str = "fp64", dt: float | None = None) -> Case:
    """Air shock on a water droplet in [0,0.02]x[0,0.01] m, extrapolation BCs.

    Fluid 1 is water (gamma 6.12, pi_inf 3.43e8 Pa, rho 1000), fluid 2 air
    (gamma 1.4, rho 1.2, p 101325).  The droplet (centre (0.008, 0.005)) is
    tanh-smoothed with smooth_coeff 0.5, i.e. its volume fraction goes from
    0.12 to 0.88 over about two cells.  The shocked air occupies x < 0.004.
    """
    gw, piw = stiffened(6.12, 3.43e8)
    ga, pia = stiffened(1.4)
    p_air, rho_air = 101325.0, 1.2
    rho2, u2, p2 = normal_shock(1.4, rho_air, p_air, mach)
    Lx, Ly = 0.02, 0.01
    bg = Patch(geometry=3, centroid=(Lx / 2, Ly / 2, 0), length=(Lx, Ly, 0),
               alpha_rho=(0.0, rho_air), alpha=(0.0, 1.0), vel=(0.0, 0.0, 0), pres=p_air)
    shocked = Patch(geometry=3, centroid=(0.002, Ly / 2, 0), length=(0.004, Ly, 0), alter_patch=(1,),
                    alpha_rho=(0.0, rho2), alpha=(0.0, 1.0), vel=(u2, 0.0, 0), pres=p2)
    drop = Patch(geometry=2, centroid=(0.008, 0.005, 0), radius=radius, smoothen=True, smooth_patch_id=1,
                 smooth_coeff=smooth_coeff, alter_patch=(1,),
                 alpha_rho=(1000.0, 0.0), alpha=(1.0, 0.0), vel=(0.0, 0.0, 0), pres=p_air)
    case = Case(m=nx - 1, n=ny - 1, x_domain=(0.0, Lx), y_domain=(0.0, Ly), dt=1.0, t_step_stop=steps,
                t_step_save=steps, num_fluids=2, time_stepper=3, weno_order=5, weno_eps=1e-16,
                bc_x=(-3, -3), bc_y=(-3, -3), gammas=(gw, ga), pi_infs=(piw, pia),
                patches=[bg, shocked, drop], precision=precision,
                name=f"shock_droplet_2d_{nx}x{ny}_M{mach:g}")
    if dt is None:
        x_cb, y_cb, _, q = preprocess.generate(case)
        dt = preprocess.max_wave_dt(case, q, cfl, x_cb, y_cb)
    return case.replace(dt=dt)


def shock_bubble_3d(N: int = 256, mach: float = 1.22, steps: int = 500, cfl: float = 0.3,
                    precision: str = "split", dt: float | None = None) -> Case:
    """Air shock on a helium sphere in the cube [-0.5, 0.5]^3 (z-extension).
    dt: None picks it from the initial state at the given CFL number (a host
    pre_process of the whole grid)."""
    gh, pih = stiffened(1.67)
    ga, pia = stiffened(1.4)
    rho2, u2, p2 = normal_shock(1.4, 1.0, 1.0, mach)
    bg = Patch(geometry=9, centroid=(0, 0, 0), length=(1.0, 1.0, 1.0),
               alpha_rho=(0.0, 1.0), alpha=(0.0, 1.0), vel=(0.0, 0.0, 0.0), pres=1.0)
    shocked = Patch(geometry=9, centroid=(-0.4, 0, 0), length=(0.2, 1.0, 1.0), alter_patch=(1,),
                    alpha_rho=(0.0, rho2), alpha=(0.0, 1.0), vel=(u2, 0.0, 0.0), pres=p2)
    bub = Patch(geometry=8, centroid=(0, 0, 0), radius=0.15, smoothen=True, smooth_patch_id=1,
                smooth_coeff=0.5, alter_patch=(1,),
                alpha_rho=(0.138, 0.0), alpha=(1.0, 0.0), vel=(0.0, 0.0, 0.0), pres=1.0)
    case = Case(m=N - 1, n=N - 1, p=N - 1, x_domain=(-0.5, 0.5), y_domain=(-0.5, 0.5), z_domain=(-0.5, 0.5),
                dt=1.0, t_step_stop=steps, t_step_save=steps, num_fluids=2, time_stepper=3, weno_order=5,
                weno_eps=1e-16, bc_x=(-3, -3), bc_y=(-3, -3), bc_z=(-3, -3), gammas=(gh, ga),
                pi_infs=(pih, pia), patches=[bg, shocked, bub], precision=precision,
                name=f"shock_bubble_3d_{N}")
    if dt is None:
        x_cb, y_cb, z_cb, q = preprocess.generate(case)
        dt = preprocess.max_wave_dt(case, q, cfl, x_cb, y_cb, z_cb)
    return case.replace(dt=dt)
