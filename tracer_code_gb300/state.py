"""Seeded synthetic initial states in the reference's array layouts.

The reference seeds tracers with gfortran's RANDOM_NUMBER (seed=1,
composition.f90:601-604), whose stream is compiler-specific; here each
tracer's two uniforms come from SplitMix64 keyed by (seed, tracer id), so a
state is reproducible on any machine.  Placement otherwise follows
initialize_tracers (composition.f90:593-639): ids run over corner control
volumes with i outermost, then k, then the tpc tracers of that volume; each
tracer sits at (i*dr, k*ds) + (U-1/2)*(dr, ds), clamped inside the walls by
dist_r/dist_s; Ttype = composition(x, z) with initial_comp=0
(initial_conditions.f90:149-158); with temperature tracers, Ttr is the
initial temperature profile at each tracer.
"""
from __future__ import annotations

import numpy as np

from .abi import Params

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(x: np.ndarray) -> np.ndarray:
    """SplitMix64 finaliser of x + golden gamma (Steele, Lea & Flood 2014)."""
    with np.errstate(over="ignore"):
        z = (x.astype(np.uint64) + _GOLDEN)
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniforms(seed: int, ids: np.ndarray, component: int) -> np.ndarray:
    """U in [0,1) with 53 random bits for (seed, id, component)."""
    key = (np.uint64(seed) << np.uint64(40)) ^ (ids.astype(np.uint64) * np.uint64(2) + np.uint64(component))
    z = splitmix64(key)
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def sizes(p: Params, nx: int | None = None, nz: int | None = None):
    nx = p.nx if nx is None else nx
    nz = p.nz if nz is None else nz
    span = p.order // 2 + 1
    return nx, nz, span


def xgrid(p: Params, r: np.ndarray) -> np.ndarray:
    """x(r) of grid.f90:1-12: arctan stretching for gridX = 1 (Ax as
    basics.f90:140), else x = r."""
    r = np.asarray(r, dtype=np.float64)
    if p.gridX == 1:
        ax = 1.0 / (np.arctan(p.spaceX * 0.5) - np.arctan(p.spaceX * -0.5))
        return p.aspect * (ax * np.arctan(p.spaceX * (r / p.aspect - 0.5)) + 0.5)
    return r


def zgrid(p: Params, s: np.ndarray, nz: int | None = None) -> np.ndarray:
    """z(s) of grid.f90:14-35: arctan stretching for gridZ = 1, boundary layers
    of nbound nodes and total thickness `thickness` for gridZ = 2, else z = s."""
    s = np.asarray(s, dtype=np.float64)
    nz = p.nz if nz is None else nz
    ds = 1.0 / nz
    if p.gridZ == 1:
        az = 1.0 / (np.arctan(p.spaceZ * 0.5) - np.arctan(p.spaceZ * -0.5))
        return az * np.arctan(p.spaceZ * (s - 0.5)) + 0.5
    if p.gridZ == 2:
        dzin = (1.0 - 2.0 * p.thickness) / (nz - 2 * p.nbound + 2)
        s1 = (p.nbound - 1) * ds
        s2 = 1.0 - s1
        scale = p.thickness / (np.exp(p.spaceZ * s1) - 1.0)
        return np.where(s < s1, scale * (np.exp(p.spaceZ * s) - 1.0),
                        np.where(s > s2, 1.0 - scale * (np.exp(-p.spaceZ * (s - 1.0)) - 1.0),
                                 p.thickness + (s - s1) * dzin / ds))
    return s


def grid_coordinates(p: Params, nx: int | None = None, nz: int | None = None):
    """Node coordinates x(i) = xgrid(i dr), i = -span..nx+span, and z(k) =
    zgrid(k ds)."""
    nx, nz, span = sizes(p, nx, nz)
    r = np.arange(-span, nx + span + 1, dtype=np.float64) * (p.aspect / nx)
    s = np.arange(-span, nz + span + 1, dtype=np.float64) * (1.0 / nz)
    return xgrid(p, r), zgrid(p, s, nz)


def initial_temperature(p: Params, nx: int | None = None, nz: int | None = None) -> np.ndarray:
    """T0 = (1 - z) + 0.01 cos(pi x) sin(pi z) at the node coordinates on
    (-span:nx+span, -span:nz+span), Fortran order (returned array has shape
    (nz+1+2span, nx+1+2span), i fastest in memory).  T(:,0)=1, T(:,nz)=0 as in
    basics.f90:230-231; ghosts are filled by enforceBCs at upload."""
    nx, nz, span = sizes(p, nx, nz)
    x, z = grid_coordinates(p, nx, nz)
    T = (1.0 - z)[:, None] + 0.01 * np.cos(np.pi * x)[None, :] * np.sin(np.pi * z)[:, None]
    T[span + 0, :] = 1.0
    T[span + nz, :] = 0.0
    return np.ascontiguousarray(T)


def initial_tracers(p: Params, seed: int = 1, nx: int | None = None, nz: int | None = None):
    """Returns (rtr, str, Ttype) for ntr = (nx+1)(nz+1)tpc tracers."""
    nx, nz, _ = sizes(p, nx, nz)
    dr = p.aspect / nx
    ds = 1.0 / nz
    tpc = p.tpc
    ntr = (nx + 1) * (nz + 1) * tpc
    ids = np.arange(ntr, dtype=np.int64)
    cell = ids // tpc
    i = cell // (nz + 1)
    k = cell % (nz + 1)
    ur = uniforms(seed, ids, 0)
    us = uniforms(seed, ids, 1)
    rcell = dr * i.astype(np.float64)
    scell = ds * k.astype(np.float64)
    r = rcell + (ur - 0.5) * dr
    s = scell + (us - 0.5) * ds
    dist_r = p.dist_factor * dr
    dist_s = p.dist_factor * ds
    r = np.where(r <= 0.0, dist_r, r)
    r = np.where(r >= p.aspect, p.aspect - dist_r, r)
    s = np.where(s <= 0.0, dist_s, s)
    s = np.where(s >= 1.0, 1.0 - dist_s, s)
    ttype = np.where(zgrid(p, s, nz) > p.dlayer, 0, 1).astype(np.int32)
    return np.ascontiguousarray(r), np.ascontiguousarray(s), np.ascontiguousarray(ttype)


def initial_composition(p: Params, nx: int | None = None, nz: int | None = None) -> np.ndarray:
    """Cnew(1, i, k) = composition(xg(i), zg(k)) (as in add_tracers,
    composition.f90:654-664): 1 in the dense layer z <= dlayer."""
    nx, nz, span = sizes(p, nx, nz)
    _, z = grid_coordinates(p, nx, nz)
    Cn = np.zeros((nz + 1 + 2 * span, nx + 1 + 2 * span, p.ntype), dtype=np.float64)
    if p.ntype > 0:
        Cn[:, :, 0] = np.where(z <= p.dlayer, 1.0, 0.0)[:, None]
    return np.ascontiguousarray(Cn)


def initial_state(p: Params, seed: int = 1, nx: int | None = None, nz: int | None = None) -> dict:
    nx, nz, span = sizes(p, nx, nz)
    T = initial_temperature(p, nx, nz)
    SF = np.zeros_like(T)
    st = {"T": T, "SF": SF, "Cnew": initial_composition(p, nx, nz)}
    if p.comp == 1 or p.tracer == 1:
        r, s, t = initial_tracers(p, seed, nx, nz)
        st["rtr"], st["str"] = r, s
        if p.comp == 1:
            st["Ttype"] = t
        if p.tracer == 1:
            st["Ttr"] = initial_tracer_temperature(xgrid(p, r), zgrid(p, s, nz))
    return st


def initial_tracer_temperature(x: np.ndarray, z: np.ndarray) -> np.ndarray:
    """Ttr = temperature(x, z) at each tracer's coordinates (initialize_tracers,
    composition.f90:630-633), with the grid's initial profile
    (1 - z) + 0.01 cos(pi x) sin(pi z)."""
    return np.ascontiguousarray((1.0 - z) + 0.01 * np.cos(np.pi * x) * np.sin(np.pi * z))
