"""
Balloon-Windkessel BOLD model (tvb_hpc/bold.py): attribute schema kept; the
engine integrates it inside the step kernel (TVBG_F_BOLD) with the
constants below, as dsl/dsl_cuda/CUDAmodels/refs/balloon.c:1-67 does.
"""

from .model import BaseModel


def _balloon_windkessel_constants():
    "Stephan et al. 2007 defaults (bold.py:24-57)."
    TAU_S = 0.65
    TAU_F = 0.41
    TAU_O = 0.98
    ALPHA = 0.32
    TE = 0.04
    V0 = 4.0
    E0 = 0.4
    EPSILON = 0.5
    NU_0 = 40.3
    R_0 = 25.0
    k1 = (4.3 * NU_0 * E0 * TE)
    k2 = (EPSILON * R_0 * E0 * TE)
    k3 = (1.0 - EPSILON)
    return {
        'RECIP_TAU_S': 1.0 / TAU_S, 'RECIP_TAU_F': 1.0 / TAU_F,
        'RECIP_TAU_O': 1.0 / TAU_O, 'RECIP_ALPHA': 1.0 / ALPHA,
        'E0': E0, 'RECIP_E0': 1.0 / E0, 'V0': V0, 'k1': k1, 'k2': k2, 'k3': k3,
    }


class BalloonWindkessel(BaseModel):
    "bold.py:60-74"
    const = _balloon_windkessel_constants()
    state = 's f v q'
    input = 'x'
    drift = (
        'x - RECIP_TAU_S * s - RECIP_TAU_F * (f - 1)',
        's',
        'RECIP_TAU_O * (f - v**RECIP_ALPHA)',
        'RECIP_TAU_O * (f * (1 - (1 - E0)**(1 / f)) * RECIP_E0'
        ' - v**RECIP_ALPHA * (q / v))'
    )
    obsrv = ('V0 * (   k1 * (1 - q     ) '
             '       + k2 * (1 - q / v ) '
             '       + k3 * (1 -     v ) )', )
    diffs = 0, 0, 0, 0

    #: fixed point with zero input: s = 0, f = v = q = 1 (initial balloon state)
    rest_state = (0.0, 1.0, 1.0, 1.0)
