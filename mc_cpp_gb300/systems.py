"""Seeded synthetic systems with the shapes of the reference's workloads.

No public dataset is involved: every system is generated from a seed.  Generated coordinates and
box lengths are rounded to 1e-6 Angstrom so that the same seed gives bitwise the same arrays on
x86 and Arm hosts even where the platform's libm differs in the last bit.

* ``argon_fcc``     Lennard-Jones argon on a jittered FCC lattice (864 atoms at 0.0213 atoms/A^3).
* ``water_box``     rigid 3-site water at 0.0334 molecules/A^3 (4096 molecules -> 12,288 atoms).
* ``argon_random``  argon on a jittered simple-cubic lattice for arbitrary atom counts.
* ``peptide_in_water``  a 40-atom flexible chain with random CHARMM-like bonded terms in water.
* ``water_chains`` / ``argon_chains``  independent chains of uneven sizes for the batched engine.

Parameters use the MDBAS conventions read by ``IO_MDBAS::read_ff`` (src/IO_MDBAS.cpp:446-467):
epsilon in kcal/mol, sigma_file = Rmin/2 / 2^(1/6) (so that the reference's pair form
4 eps_i eps_j [((s_i+s_j)/r)^12 - ((s_i+s_j)/r)^6] equals CHARMM's), argon sigma_file = 3.405/2.
"""
from __future__ import annotations

import math
from typing import List

import numpy as np

from .mdbas import MoveSpec, System

__all__ = ["argon_fcc", "argon_random", "water_box", "peptide_in_water", "water_chains",
           "water_chain_specs", "argon_chains", "shard_chains", "TWO_SIXTH", "WATER"]

TWO_SIXTH = 2.0 ** (1.0 / 6.0)
# rigid 3-site water (config "water box"): O-H 0.9572 A, H-O-H 104.52 deg
WATER = dict(roh=0.9572, theta=104.52, qO=-0.834, qH=0.417, epsO=0.1521, rminO=1.7682,
             epsH=0.046, rminH=0.2245, mO=15.9994, mH=1.008)


def _q(a):
    return np.round(np.asarray(a, dtype=np.float64) * 1e6) / 1e6


def _wrap(v, L):
    # the reference keeps coordinates wrapped into [-L/2, L/2] (Move.hpp:48,140)
    return v - L * np.round(v / L)


def _base(natom, x, y, z, **kw) -> System:
    return System(natom=natom, x=_q(x), y=_q(y), z=_q(z), **kw)


def argon_fcc(ncell: int = 6, density: float = 0.0213, jitter: float = 0.1, seed: int = 1,
              temp: float = 120.0, dmax: float = 0.2) -> System:
    """Argon on a perturbed FCC lattice, single-atom translation moves (the small plain workload)."""
    rng = np.random.default_rng(seed)
    n = 4 * ncell ** 3
    L = float(_q((n / density) ** (1.0 / 3.0)))
    a = L / ncell
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    cells = np.array([[i, j, k] for i in range(ncell) for j in range(ncell) for k in range(ncell)], float)
    pos = (cells[:, None, :] + basis[None, :, :]).reshape(-1, 3) * a - L / 2 + a / 4
    pos += rng.uniform(-jitter, jitter, size=pos.shape)
    pos = _wrap(pos, L)
    return _base(n, pos[:, 0], pos[:, 1], pos[:, 2],
                 q=np.zeros(n), eps=np.full(n, 0.2381), sig=np.full(n, 3.405 / 2), eps14=np.zeros(n),
                 sig14=np.zeros(n), mass=np.full(n, 39.948), frozen=np.zeros(n, np.uint8),
                 resid=np.arange(1, n + 1, dtype=np.int32), resname=["ARR"] * n, atname=["AR"] * n,
                 segname=["ARG"] * n, atom_type=np.ones(n, np.int32), pbc_type="cubic", box=(L, L, L),
                 cut_mode="switch", cutoff=12.0, cuton=10.0, dcut=2.0, temp=temp,
                 moves=[MoveSpec("trn", "atom", "all", "", dmax, 50.0, 0)])


def argon_random(n: int, density: float, seed: int, temp: float = 120.0, dmax: float = 0.2,
                 jitter: float = 0.25) -> System:
    """Argon at an arbitrary atom count: a random subset of a simple-cubic lattice, jittered."""
    rng = np.random.default_rng(seed)
    L = float(_q((n / density) ** (1.0 / 3.0)))
    m = int(math.ceil(n ** (1.0 / 3.0)))
    a = L / m
    sites = np.array([[i, j, k] for i in range(m) for j in range(m) for k in range(m)], float)
    pick = np.sort(rng.permutation(len(sites))[:n])
    pos = sites[pick] * a - L / 2 + a / 2 + rng.uniform(-jitter, jitter, size=(n, 3))
    pos = _wrap(pos, L)
    return _base(n, pos[:, 0], pos[:, 1], pos[:, 2],
                 q=np.zeros(n), eps=np.full(n, 0.2381), sig=np.full(n, 3.405 / 2), eps14=np.zeros(n),
                 sig14=np.zeros(n), mass=np.full(n, 39.948), frozen=np.zeros(n, np.uint8),
                 resid=np.arange(1, n + 1, dtype=np.int32), resname=["ARR"] * n, atname=["AR"] * n,
                 segname=["ARG"] * n, atom_type=np.ones(n, np.int32), pbc_type="cubic", box=(L, L, L),
                 cut_mode="switch", cutoff=12.0, cuton=10.0, dcut=2.0, temp=temp,
                 moves=[MoveSpec("trn", "atom", "all", "", dmax, 50.0, 0)])


def _random_rotations(rng, n):
    # uniform random rotation matrices from unit quaternions (Shoemake's method)
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    a, b = np.sqrt(1 - u1), np.sqrt(u1)
    qw, qx = a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2)
    qy, qz = b * np.sin(2 * np.pi * u3), b * np.cos(2 * np.pi * u3)
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (qy * qy + qz * qz); R[:, 0, 1] = 2 * (qx * qy - qz * qw); R[:, 0, 2] = 2 * (qx * qz + qy * qw)
    R[:, 1, 0] = 2 * (qx * qy + qz * qw); R[:, 1, 1] = 1 - 2 * (qx * qx + qz * qz); R[:, 1, 2] = 2 * (qy * qz - qx * qw)
    R[:, 2, 0] = 2 * (qx * qz - qy * qw); R[:, 2, 1] = 2 * (qy * qz + qx * qw); R[:, 2, 2] = 1 - 2 * (qx * qx + qy * qy)
    return R


def _water_geometry():
    w = WATER
    h = math.radians(w["theta"]) / 2
    return np.array([[0.0, 0.0, 0.0],
                     [w["roh"] * math.sin(h), 0.0, w["roh"] * math.cos(h)],
                     [-w["roh"] * math.sin(h), 0.0, w["roh"] * math.cos(h)]])


def _water_topology(nmol: int, first_atom: int = 0, first_res: int = 1):
    w = WATER
    n = 3 * nmol
    o = first_atom + 3 * np.arange(nmol, dtype=np.int32)
    bonds = np.stack([np.stack([o, o + 1], 1), np.stack([o, o + 2], 1)], 1).reshape(-1, 2)
    angles = np.stack([o + 1, o, o + 2], 1)
    sigO, sigH = w["rminO"] / TWO_SIXTH, w["rminH"] / TWO_SIXTH
    return dict(
        q=np.tile([w["qO"], w["qH"], w["qH"]], nmol), eps=np.tile([w["epsO"], w["epsH"], w["epsH"]], nmol),
        sig=np.tile([sigO, sigH, sigH], nmol), eps14=np.tile([w["epsO"], w["epsH"], w["epsH"]], nmol),
        sig14=np.tile([sigO, sigH, sigH], nmol), mass=np.tile([w["mO"], w["mH"], w["mH"]], nmol),
        frozen=np.zeros(n, np.uint8), resid=np.repeat(np.arange(first_res, first_res + nmol, dtype=np.int32), 3),
        resname=["TIP3"] * n, atname=["OH2", "H1", "H2"] * nmol, segname=["WAT"] * n,
        atom_type=np.tile(np.array([2, 3, 3], np.int32), nmol),
        bonds=bonds.astype(np.int32), bond_type=np.zeros(len(bonds), np.int32),
        bond_k=np.full(len(bonds), 450.0), bond_r0=np.full(len(bonds), w["roh"]), bond_beta=np.zeros(len(bonds)),
        angles=angles.astype(np.int32), angle_type=np.zeros(nmol, np.int32), angle_k=np.full(nmol, 55.0),
        angle_theta0=np.full(nmol, w["theta"]))


def _water_positions(rng, nmol, L, jitter=0.2, exclude=None, min_dist=2.6):
    m = int(math.ceil(nmol ** (1.0 / 3.0)))
    while True:
        a = L / m
        sites = np.array([[i, j, k] for i in range(m) for j in range(m) for k in range(m)], float) * a - L / 2 + a / 2
        if exclude is not None and len(exclude):
            d = sites[:, None, :] - exclude[None, :, :]
            d -= L * np.round(d / L)
            ok = (np.sqrt((d * d).sum(-1)).min(1) > min_dist)
            sites = sites[ok]
        if len(sites) >= nmol:
            break
        m += 1
    pick = np.sort(rng.permutation(len(sites))[:nmol])
    centers = sites[pick] + rng.uniform(-jitter, jitter, size=(nmol, 3))
    R = _random_rotations(rng, nmol)
    geo = _water_geometry()
    pos = centers[:, None, :] + np.einsum("nij,aj->nai", R, geo)
    return _wrap(pos.reshape(-1, 3), L)


def water_box(nmol: int = 4096, density: float = 0.0334, seed: int = 2, temp: float = 298.0,
              L: float = None, dmax_trn: float = 0.15, dmax_rot: float = 15.0) -> System:
    """Rigid 3-site water, random orientations on a jittered cubic lattice (residue moves)."""
    rng = np.random.default_rng(seed)
    L = float(_q(L if L is not None else (nmol / density) ** (1.0 / 3.0)))
    pos = _water_positions(rng, nmol, L)
    top = _water_topology(nmol)
    return _base(3 * nmol, pos[:, 0], pos[:, 1], pos[:, 2], **top, pbc_type="cubic", box=(L, L, L),
                 cut_mode="switch", cutoff=12.0, cuton=10.0, dcut=2.0, temp=temp,
                 moves=[MoveSpec("trn", "residue", "residue_name", "TIP3", dmax_trn, 50.0, 0),
                        MoveSpec("rot", "residue", "residue_name", "TIP3", dmax_rot, 50.0, 0)])


def peptide_in_water(nchain: int = 40, nwat: int = 6000, L: float = 56.4, seed: int = 4,
                     temp: float = 300.0) -> System:
    """A flexible 40-atom chain with random CHARMM-like terms, solvated in rigid water.

    Bonds k in [200,400] kcal/mol/A^2, angles, Urey-Bradley, periodic dihedrals n in {1,2,3}
    (cosine form), harmonic impropers; charges ~N(0,0.3) shifted to sum 0; eps in [0.02,0.2];
    Rmin/2 in [1.0,2.2]; 1-4 pairs use eps14 = eps/2, sigma14 = sigma.
    """
    rng = np.random.default_rng(seed)
    L = float(_q(L))
    # self-avoiding-ish random walk with 1.53 A bonds and ~111 deg angles
    pos = [np.zeros(3)]
    d = np.array([1.0, 0.0, 0.0])
    while len(pos) < nchain:
        v = rng.normal(size=3)
        v -= v.dot(d) * d
        v /= np.linalg.norm(v)
        ang = math.radians(180.0 - 111.0)
        nd = math.cos(ang) * d + math.sin(ang) * v
        cand = pos[-1] + 1.53 * nd
        if len(pos) > 3 and np.min(np.linalg.norm(np.array(pos[:-2]) - cand, axis=1)) < 2.6:
            continue
        pos.append(cand)
        d = nd
    pep = np.array(pos)
    pep -= pep.mean(0)
    pep = _q(_wrap(pep, L))
    nb = nchain - 1
    bonds = np.stack([np.arange(nb), np.arange(1, nchain)], 1).astype(np.int32)

    def dist(i, j):
        v = pep[j] - pep[i]
        v -= L * np.round(v / L)
        return float(np.linalg.norm(v))

    def angle(i, j, k):
        a, b = pep[i] - pep[j], pep[k] - pep[j]
        return math.degrees(math.acos(float(a.dot(b) / np.linalg.norm(a) / np.linalg.norm(b))))

    angles = np.stack([np.arange(nchain - 2), np.arange(1, nchain - 1), np.arange(2, nchain)], 1).astype(np.int32)
    dihe = np.stack([np.arange(nchain - 3), np.arange(1, nchain - 2), np.arange(2, nchain - 1),
                     np.arange(3, nchain)], 1).astype(np.int32)
    impr_idx = np.arange(1, nchain - 2, 6)
    impr = np.stack([impr_idx, impr_idx - 1, impr_idx + 1, impr_idx + 2], 1).astype(np.int32)
    ub_idx = np.arange(0, nchain - 2, 3)
    ub = np.stack([ub_idx, ub_idx + 2], 1).astype(np.int32)
    q = rng.normal(0.0, 0.3, size=nchain)
    q = _q(q - q.mean())
    q[-1] = _q(q[-1] - q.sum())
    eps = _q(rng.uniform(0.02, 0.2, nchain))
    sig = _q(rng.uniform(1.0, 2.2, nchain) / TWO_SIXTH)
    pep_kw = dict(
        q=q, eps=eps, sig=sig, eps14=_q(eps / 2), sig14=sig.copy(), mass=np.full(nchain, 12.011),
        frozen=np.zeros(nchain, np.uint8), resid=np.ones(nchain, np.int32), resname=["PEP"] * nchain,
        atname=["C%d" % i for i in range(nchain)], segname=["PEP"] * nchain, atom_type=np.ones(nchain, np.int32),
        bonds=bonds, bond_type=np.zeros(nb, np.int32), bond_k=_q(rng.uniform(200, 400, nb)),
        bond_r0=_q([dist(i, i + 1) for i in range(nb)]), bond_beta=np.zeros(nb),
        ub=ub, ub_k=_q(rng.uniform(5, 30, len(ub))), ub_r0=_q([dist(i, i + 2) for i in ub_idx]),
        angles=angles, angle_type=np.zeros(len(angles), np.int32), angle_k=_q(rng.uniform(30, 80, len(angles))),
        angle_theta0=_q([angle(*t) for t in angles]),
        dihedrals=dihe, dihe_type=np.ones(len(dihe), np.int32),
        dihe_order=rng.integers(1, 4, len(dihe)).astype(np.int32), dihe_k=_q(rng.uniform(0.1, 2.0, len(dihe))),
        dihe_phi0=_q(rng.choice([0.0, 180.0], len(dihe))), dihe_mult=None,
        impropers=impr, impr_type=np.full(len(impr), 2, np.int32), impr_order=np.ones(len(impr), np.int32),
        impr_k=_q(rng.uniform(5, 50, len(impr))), impr_phi0=np.zeros(len(impr)), impr_mult=np.ones(len(impr)))
    pep_kw["dihe_mult"] = pep_kw["dihe_order"].astype(np.float64)
    wpos = _water_positions(rng, nwat, L, exclude=pep)
    top = _water_topology(nwat, first_atom=nchain, first_res=2)
    n = nchain + 3 * nwat
    cat = lambda a, b: np.concatenate([a, b])
    kw = {}
    for k in ("q", "eps", "sig", "eps14", "sig14", "mass", "frozen", "resid", "atom_type"):
        kw[k] = cat(pep_kw[k], top[k])
    for k in ("resname", "atname", "segname"):
        kw[k] = pep_kw[k] + top[k]
    kw["bonds"] = cat(pep_kw["bonds"], top["bonds"]).astype(np.int32)
    for k in ("bond_type", "bond_k", "bond_r0", "bond_beta"):
        kw[k] = cat(pep_kw[k], top[k])
    kw["angles"] = cat(pep_kw["angles"], top["angles"]).astype(np.int32)
    for k in ("angle_type", "angle_k", "angle_theta0"):
        kw[k] = cat(pep_kw[k], top[k])
    for k in ("ub", "ub_k", "ub_r0", "dihedrals", "dihe_type", "dihe_order", "dihe_k", "dihe_phi0", "dihe_mult",
              "impropers", "impr_type", "impr_order", "impr_k", "impr_phi0", "impr_mult"):
        kw[k] = pep_kw[k]
    allpos = np.concatenate([pep, wpos])
    return _base(n, allpos[:, 0], allpos[:, 1], allpos[:, 2], **kw, pbc_type="cubic", box=(L, L, L),
                 cut_mode="switch", cutoff=12.0, cuton=10.0, dcut=2.0, temp=temp,
                 moves=[MoveSpec("trn", "atom", "residue_name", "PEP", 0.1, 50.0, 0),
                        MoveSpec("trn", "residue", "residue_name", "TIP3", 0.15, 50.0, 0),
                        MoveSpec("rot", "residue", "residue_name", "TIP3", 15.0, 50.0, 0)])


def water_chain_specs(nchains: int = 256, nmin: int = 512, nmax: int = 8192, tmin: float = 280.0,
                      tmax: float = 360.0, seed: int = 3):
    """(molecules, seed, temperature) of each chain of water_chains, without building the boxes."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(math.log(nmin), math.log(nmax), nchains)).astype(np.int64)
    sizes = np.clip(sizes, nmin, nmax)
    temps = _q(rng.uniform(tmin, tmax, nchains))
    seeds = rng.integers(1, 2 ** 31 - 1, nchains)
    return [(int(n), int(s), float(t)) for n, s, t in zip(sizes, seeds, temps)]


def water_chains(nchains: int = 256, nmin: int = 512, nmax: int = 8192, density: float = 0.0334,
                 tmin: float = 280.0, tmax: float = 360.0, seed: int = 3, only=None) -> List[System]:
    """Independent water boxes of log-uniform molecule counts and uniform temperatures; `only`
    (indices into the nchains specs) builds a subset, in that order."""
    specs = water_chain_specs(nchains, nmin, nmax, tmin, tmax, seed)
    pick = range(nchains) if only is None else only
    return [water_box(specs[i][0], density, specs[i][1], specs[i][2]) for i in pick]


def argon_chains(nchains: int = 1024, nmin: int = 500, nmax: int = 2000, rho_min: float = 0.015,
                 rho_max: float = 0.025, tmin: float = 90.0, tmax: float = 150.0, seed: int = 5) -> List[System]:
    """Independent argon boxes: N ~ U{500..2000}, density ~ U[0.015,0.025], T ~ U[90,150] K."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(nmin, nmax + 1, nchains)
    rhos = rng.uniform(rho_min, rho_max, nchains)
    temps = _q(rng.uniform(tmin, tmax, nchains))
    seeds = rng.integers(1, 2 ** 31 - 1, nchains)
    return [argon_random(int(n), float(r), int(s), float(t)) for n, r, s, t in zip(sizes, rhos, seeds, temps)]


def shard_chains(weights, world: int):
    """Greedy longest-first partition of independent chains over `world` ranks: chains in order
    of decreasing weight (atoms), each to the rank with the least total so far (lowest rank on a
    tie).  Returns each rank's chain indices, ascending.  The largest total exceeds the smallest by
    at most the largest weight."""
    if world < 1:
        raise ValueError("world must be >= 1")
    w = [float(v) for v in weights]
    order = sorted(range(len(w)), key=lambda i: (-w[i], i))
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        load[r] += w[i]
        parts[r].append(i)
    return [sorted(p) for p in parts]
