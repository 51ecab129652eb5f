"""Small cases shared by the tests (sizes the oracle finishes in seconds)."""
from __future__ import annotations

from tracer_code_gb300.abi import Params, config_1024x256, config_plain_128, default_params
from tracer_code_gb300 import state


def case_1024_like(nx: int = 128, nz: int = 32, tpc: int = 3, grids: int = 4, Ra: float = 1.0e5,
                   visT: float = 100.0) -> Params:
    """The 1024x256 case's setup (aspect 4, B=0.8, T- and C-dependent
    viscosity, dense layer z<0.1) on a smaller grid.  At these sizes the
    full contrast (visT=1e4) at Ra=1e7 advects wall tracers across the side
    walls in the start-up transient (the reference stops there too), so the
    parity cases use a contrast of 100 and Ra=1e5 by default."""
    p = config_1024x256()
    p.nx, p.nz, p.tpc, p.grids = nx, nz, tpc, grids
    p.RaT = Ra
    p.RaC[0] = 0.8 * Ra
    p.visT = visT
    return p


def case_128_like(nx: int = 32, nz: int = 32, tpc: int = 4, grids: int = 4) -> Params:
    """The 128x128 isoviscous physics (Ra=1e5, B=0.5) on a smaller grid."""
    p = config_plain_128()
    p.nx, p.nz, p.tpc, p.grids = nx, nz, tpc, grids
    return p


def fresh_state(p: Params, seed: int = 1) -> dict:
    return state.initial_state(p, seed=seed)
