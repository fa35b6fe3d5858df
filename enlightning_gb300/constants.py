"""Physical constants and default parameters of the time advance.

Values follow the reference's input file (input.txt:2-59) except where the
synthetic workloads override them (rho0 = 1.2, gamma1 = 1.4).  tau_n / tau_o
are derived exactly as enlightning.C:217-234 does.
"""
from __future__ import annotations

import math

NEQU = 5          # enlightning.h:48
CELLG = 3         # enlightning.C:68 (ghost width)
REFLECT = 10      # enlightning.C:64
ABSORB = 20       # enlightning.C:65

# SSP-RK3 coefficients, input.txt:130-133 (exact decimals as written there).
RK3_ALPHA1 = (1.0, 0.75, 0.3333333333)
RK3_ALPHA2 = (0.0, 0.25, 0.6666666667)
RK3_BETA = (1.0, 0.25, 0.6666666667)

VARIANTS = (
    "hybrid_high_llf", "hybrid_high", "hybrid_low_llf", "hybrid_low",
    "weno_high_llf", "weno_high", "weno_low_llf", "weno_low", "drp",
)


def relaxation_times(p0: float, T0: float, RH: float) -> tuple[float, float]:
    """tau_n, tau_o of enlightning.C:217-234 (T_ref = T0, p_ref = p0)."""
    PI = 3.14159265358979323846264338
    T_ref, p_ref = T0, p0
    zeta = (10.79586 * (1 - (273.16 / T0)) - 5.02808 * math.log10(T0 / 273.16)
            + (1.50474e-4) * (1 - math.pow(10, (-8.29692 * ((T0 / 273.16) - 1))))
            - (4.2873e-4) * (1 - math.pow(10, (-4.76955 * ((273.16 / T0) - 1))))
            - 2.2195983)
    p_vp = p_ref * math.pow(10, zeta)
    h = (RH * p_vp) / p0
    eta = 4.17 * (math.pow(T_ref / T0, 1.0 / 3.0) - 1)
    f_n = (p0 / p_ref) * (math.pow((T_ref / T0), 0.5) * (9 + 280 * h * math.exp(-eta)))
    f_o = (p0 / p_ref) * (24 + (4.04e4) * h * ((0.02 + h) / (0.391 + h)))
    return 1 / (2 * PI * f_n), 1 / (2 * PI * f_o)


def default_params(**over) -> dict:
    """Parameter dictionary consumed by the host strategy, the oracle and the tests."""
    p = dict(
        weno_alpha=360.0, alpha=360.0, c=343.0, gamma1=1.4, p0=101325.0, RH=20.0, T0=293.16,
        c_lr=0.0, rho0=1.2, R=287.06, c_p=1010.0, T_star_n=3352.0, T_star_o=2239.0,
        mu=1.846e-5, muB=1.1076e-5, kappa=0.02624, c_v=720.4, R_tilde=8314.32, M=28.9644,
        tol=(1.5, 1e-2, 5e-3), cfl=0.5, bc_absorb_width=1e-2,
    )
    p.update(over)
    p["alpha"] = p["weno_alpha"]
    p["tau_n"], p["tau_o"] = relaxation_times(p["p0"], p["T0"], p["RH"])
    return p
