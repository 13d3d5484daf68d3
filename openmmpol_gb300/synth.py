"""Seeded synthetic polarizable systems written as revision-3 ``.mmp`` files.

Workloads (sizes and value distributions of the benchmark configurations):

* ``water_cluster(n)``: AMOEBA water on a jittered cubic lattice at
  0.0334 molecules/A^3 (spacing 3.104 A), +-0.25 A uniform jitter per axis,
  uniformly random orientations (random unit quaternion), O-H 0.9572 A,
  H-O-H 104.52 deg; lattice cells are filled in x-fastest order from a cube
  of ceil(n^(1/3)) cells per side.  A chosen guard re-draws the orientation of
  a molecule whose atoms come closer than 1.0 A to another molecule.
  AMOEBA water parameters are those of Tinker types 349/350 as they appear
  in the reference's tests/1ubq/input_AMOEBA.mmp (local-frame multipoles,
  polarizabilities 0.837 / 0.496 A^3, bisector frame on O, z-then-x on H,
  one polarization group per molecule); Thole a = 0.39 is set by the loader.
* ``chain_system()``: Wang-AL (AMBER-style) system of self-avoiding random
  walk chains (bond 1.53 A, no site closer than 2.0 A to an earlier one)
  embedded in water at 0.0334 molecules/A^3; chain charges U(-0.6, 0.6) e,
  polarizabilities U(0.4, 1.5) A^3; a chosen neutral water model
  (O -0.8 e / H +0.4 e, 0.837 / 0.496 A^3).  Non-AMOEBA .mmp polarizabilities
  are read in atomic units (the loader converts only AMOEBA ones,
  src/mod_inputloader.F90:205-209), so they are written in bohr^3.
* ``point_charge_field()``: field of 30 point charges U(-0.5, 0.5) e placed
  uniformly in a 6 A ball at the box centre, at least 1.0 A from every site:
  E_i = sum_c q_c (r_i - r_c) / |r_i - r_c|^3 in atomic units (the formula of
  src/mod_qm_helper.F90:373-389).

Everything is deterministic in the seed.
"""
from __future__ import annotations

import math
import os

import numpy as np

ANG2AU = 1.8897261245650
WATER_DENSITY = 0.0334  # molecules / A^3

# AMOEBA water, local frame: q, px, py, pz, Qxx, Qxy, Qyy, Qxz, Qyz, Qzz
_O_MULT = [-0.51966, 0.0, 0.0, 0.14279, 0.37928, 0.0, -0.41809, 0.0, 0.0, 0.03881]
_H_MULT = [0.25983, -0.03859, 0.0, -0.05818, -0.03673, 0.0, -0.10739, -0.00203, 0.0, 0.14412]
_O_POL, _H_POL = 0.837, 0.496
_ROH, _HOH = 0.9572, math.radians(104.52)


class MMPSystem:
    """Plain arrays of one system, in the units of the .mmp file (A)."""

    def __init__(self, amoeba, coords, mult, pol, bonds, groups=None, frames=None, z=None):
        self.amoeba = amoeba
        self.coords = np.asarray(coords, dtype=np.float64)
        self.mult = np.asarray(mult, dtype=np.float64)
        self.pol = np.asarray(pol, dtype=np.float64)
        self.bonds = bonds            # int array [mm, 8], 1-based, 0 = none
        self.groups = groups          # list of 1-based member lists per atom (AMOEBA)
        self.frames = frames          # int array [mm, 4] (frame, iz, ix, iy), 1-based
        self.z = z if z is not None else np.ones(len(self.coords), dtype=np.int32)

    @property
    def mm_atoms(self):
        return len(self.coords)

    def box_center(self):
        return 0.5 * (self.coords.min(axis=0) + self.coords.max(axis=0))


def _random_rotations(rng, n):
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - z * w)
    R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w)
    R[:, 2, 1] = 2 * (y * z + x * w)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def _water_atoms(O, R):
    s, c = math.sin(_HOH / 2), math.cos(_HOH / 2)
    h1 = np.array([_ROH * s, 0.0, _ROH * c])
    h2 = np.array([-_ROH * s, 0.0, _ROH * c])
    H1 = O + R @ h1
    H2 = O + R @ h2
    return H1, H2


def water_cluster(n_waters: int, seed: int = 1, jitter: float = 0.25, guard: float = 1.0,
                  origin=(0.0, 0.0, 0.0)) -> MMPSystem:
    rng = np.random.default_rng(seed)
    a = (1.0 / WATER_DENSITY) ** (1.0 / 3.0)
    side = int(math.ceil(n_waters ** (1.0 / 3.0) - 1e-9))
    idx = np.arange(n_waters)
    cell = np.stack([idx % side, (idx // side) % side, idx // (side * side)], axis=1)
    O = cell * a + rng.uniform(-jitter, jitter, size=(n_waters, 3)) + np.asarray(origin)
    R = _random_rotations(rng, n_waters)
    H1, H2 = _water_atoms(O, R)
    # orientation guard: redraw molecules with an atom closer than `guard` to
    # an atom of a lattice neighbour (intramolecular pairs excluded)
    lookup = -np.ones((side + 2, side + 2, side + 2), dtype=np.int64)
    lookup[cell[:, 0] + 1, cell[:, 1] + 1, cell[:, 2] + 1] = idx
    offs = [(i, j, k) for i in (-1, 0, 1) for j in (-1, 0, 1) for k in (-1, 0, 1) if (i, j, k) > (0, 0, 0)]
    for _ in range(200):
        atoms = np.stack([O, H1, H2], axis=1)  # [n,3,3]
        bad = np.zeros(n_waters, dtype=bool)
        for o in offs:
            nb = lookup[cell[:, 0] + 1 + o[0], cell[:, 1] + 1 + o[1], cell[:, 2] + 1 + o[2]]
            has = nb >= 0
            if not has.any():
                continue
            A = atoms[has][:, :, None, :]
            B = atoms[nb[has]][:, None, :, :]
            d = np.linalg.norm(A - B, axis=-1).min(axis=(1, 2))
            clash = d < guard
            bad[np.nonzero(has)[0][clash]] = True
        if not bad.any():
            break
        nbad = int(bad.sum())
        R[bad] = _random_rotations(rng, nbad)
        H1[bad], H2[bad] = _water_atoms(O[bad], R[bad])
    coords = np.empty((3 * n_waters, 3))
    coords[0::3], coords[1::3], coords[2::3] = O, H1, H2
    mult = np.tile(np.array([_O_MULT, _H_MULT, _H_MULT]), (n_waters, 1))
    pol = np.tile(np.array([_O_POL, _H_POL, _H_POL]), n_waters)
    base = 3 * np.arange(n_waters) + 1  # 1-based O index
    bonds = np.zeros((3 * n_waters, 8), dtype=np.int64)
    bonds[0::3, 0], bonds[0::3, 1] = base + 1, base + 2
    bonds[1::3, 0] = base
    bonds[2::3, 0] = base
    frames = np.zeros((3 * n_waters, 4), dtype=np.int64)
    frames[0::3] = np.stack([np.full(n_waters, 2), base + 1, base + 2, np.zeros(n_waters, np.int64)], 1)
    frames[1::3] = np.stack([np.ones(n_waters, np.int64), base, base + 2, np.zeros(n_waters, np.int64)], 1)
    frames[2::3] = np.stack([np.ones(n_waters, np.int64), base, base + 1, np.zeros(n_waters, np.int64)], 1)
    groups = np.repeat(np.stack([base, base + 1, base + 2], axis=1), 3, axis=0)
    z = np.tile(np.array([8, 1, 1], dtype=np.int32), n_waters)
    return MMPSystem(True, coords, mult, pol, bonds, groups=groups, frames=frames, z=z)


def chain_system(n_chains: int = 150, chain_len: int = 200, n_waters: int = 10000, seed: int = 3,
                 bond: float = 1.53, min_dist: float = 2.0, water_clear: float = 2.5) -> MMPSystem:
    # box sized so that the waters fill what the chains leave at water
    # density; grown by 4 % steps (same seed) until every water fits
    n_chain_sites = n_chains * chain_len
    L0 = ((n_waters + 0.5 * n_chain_sites) / WATER_DENSITY) ** (1.0 / 3.0)
    for grow in range(40):
        s = _chain_system_in_box(L0 * 1.04 ** grow, n_chains, chain_len, n_waters, seed, bond,
                                 min_dist, water_clear)
        if s is not None:
            return s
    raise RuntimeError("could not fit the waters around the chains")


def _chain_system_in_box(L, n_chains, chain_len, n_waters, seed, bond, min_dist, water_clear):
    rng = np.random.default_rng(seed)
    n_chain_sites = n_chains * chain_len
    cs = min_dist
    ncell = max(1, int(L / cs))
    grid: dict = {}

    def cell_of(p):
        return tuple(np.minimum((p / L * ncell).astype(int), ncell - 1))

    def free(p, prev=None):
        # `prev` is the bonded predecessor (1.53 A away): exempt from the test
        if np.any(p < 0) or np.any(p >= L):
            return False
        c = cell_of(p)
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    for q in grid.get((c[0] + dx, c[1] + dy, c[2] + dz), ()):
                        if q is not prev and np.sum((q - p) ** 2) < min_dist * min_dist:
                            return False
        return True

    def add(p):
        grid.setdefault(cell_of(p), []).append(p)

    chains = []
    while len(chains) < n_chains:
        for _attempt in range(100):
            p0 = rng.uniform(0.0, L, 3)
            if free(p0):
                break
        walk = [p0]
        placed = [p0]
        add(p0)
        ok = True
        while len(walk) < chain_len:
            for _t in range(50):
                v = rng.standard_normal(3)
                p = walk[-1] + bond * v / np.linalg.norm(v)
                if free(p, walk[-1]):
                    walk.append(p)
                    add(p)
                    placed.append(p)
                    break
            else:
                ok = False
                break
        if ok:
            chains.append(np.array(walk))
        else:  # remove this chain's sites and retry
            for p in placed:
                grid[cell_of(p)] = [q for q in grid[cell_of(p)] if q is not p]
    chain_xyz = np.concatenate(chains)
    # waters on the lattice points that keep clear of the chains
    a = (1.0 / WATER_DENSITY) ** (1.0 / 3.0)
    side = int(L / a)
    g = np.stack(np.meshgrid(np.arange(side), np.arange(side), np.arange(side), indexing="ij"), -1).reshape(-1, 3)
    g = g[:, ::-1]  # x fastest
    O = (g + 0.5) * a + rng.uniform(-0.25, 0.25, size=g.shape)
    keep = np.ones(len(O), dtype=bool)
    cc = np.floor(chain_xyz / a).astype(int)
    occupied = {}
    for i, c in enumerate(map(tuple, cc)):
        occupied.setdefault(c, []).append(i)
    oc = np.floor(O / a).astype(int)
    for k in range(len(O)):
        c = oc[k]
        near = []
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    near.extend(occupied.get((c[0] + dx, c[1] + dy, c[2] + dz), ()))
        if near and np.min(np.linalg.norm(chain_xyz[near] - O[k], axis=1)) < water_clear:
            keep[k] = False
    O = O[keep]
    if len(O) < n_waters:
        return None
    O = O[:n_waters]
    R = _random_rotations(rng, n_waters)
    H1, H2 = _water_atoms(O, R)
    nc = n_chain_sites
    mm = nc + 3 * n_waters
    coords = np.empty((mm, 3))
    coords[:nc] = chain_xyz
    coords[nc::3], coords[nc + 1::3], coords[nc + 2::3] = O, H1, H2
    q = np.empty(mm)
    q[:nc] = rng.uniform(-0.6, 0.6, nc)
    q[nc::3], q[nc + 1::3], q[nc + 2::3] = -0.8, 0.4, 0.4
    pol_a3 = np.empty(mm)
    pol_a3[:nc] = rng.uniform(0.4, 1.5, nc)
    pol_a3[nc::3], pol_a3[nc + 1::3], pol_a3[nc + 2::3] = _O_POL, _H_POL, _H_POL
    bonds = np.zeros((mm, 8), dtype=np.int64)
    for c in range(n_chains):
        s0 = c * chain_len
        for i in range(chain_len):
            k = 0
            if i > 0:
                bonds[s0 + i, k] = s0 + i  # 1-based index of the previous site
                k += 1
            if i < chain_len - 1:
                bonds[s0 + i, k] = s0 + i + 2
    base = nc + 3 * np.arange(n_waters) + 1
    bonds[nc::3, 0], bonds[nc::3, 1] = base + 1, base + 2
    bonds[nc + 1::3, 0] = base
    bonds[nc + 2::3, 0] = base
    z = np.full(mm, 6, dtype=np.int32)
    z[nc::3], z[nc + 1::3], z[nc + 2::3] = 8, 1, 1
    return MMPSystem(False, coords, q[:, None], pol_a3 * ANG2AU ** 3, bonds, z=z)


def write_mmp(path: str, s: MMPSystem) -> str:
    """Write a revision-3 .mmp file readable by OpenMMPol's loader
    (src/mod_inputloader.F90:15-257)."""
    mm = s.mm_atoms
    lines = ["3", "0", "0", "1" if s.amoeba else "0", "0"] + ["0"] * 17 + [str(mm), "0"]
    lines += [str(int(v)) for v in s.z]
    lines += ["%.10f %.10f %.10f" % tuple(c) for c in s.coords]
    lines += ["1"] * mm
    fmt = " ".join(["%.8f"] * s.mult.shape[1])
    lines += [fmt % tuple(m) for m in s.mult]
    lines += ["%.8f" % p for p in s.pol]
    lines += [" ".join(str(int(v)) for v in b) for b in s.bonds]
    if s.amoeba:
        for g in s.groups:
            members = [str(int(v)) for v in g]
            lines.append(" ".join(members) + " %d*0" % (120 - len(members)))
        lines += ["%d %d %d %d" % tuple(f) for f in s.frames]
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    with open(path, "w") as f:
        f.write("\n".join(lines))
        f.write("\n")
    return path


def point_charge_field(cpol_bohr, center_ang, n_charges: int = 30, seed: int = 1, radius: float = 6.0,
                       guard: float = 1.0, qmax: float = 0.5, all_sites_bohr=None):
    """Field [npol, 3] (a.u.) of n random point charges; returns (field, charges, positions_bohr)."""
    rng = np.random.default_rng(seed)
    sites = np.asarray(all_sites_bohr if all_sites_bohr is not None else cpol_bohr)
    c0 = np.asarray(center_ang) * ANG2AU
    rad, grd = radius * ANG2AU, guard * ANG2AU
    pos, q = [], []
    # only sites within radius + guard of the centre can violate the guard
    near = sites[np.linalg.norm(sites - c0, axis=1) < rad + grd + 1e-9]
    while len(pos) < n_charges:
        v = rng.uniform(-1.0, 1.0, 3)
        if np.dot(v, v) > 1.0:
            continue
        p = c0 + rad * v
        if len(near) and np.min(np.linalg.norm(near - p, axis=1)) < grd:
            continue
        pos.append(p)
        q.append(rng.uniform(-qmax, qmax))
    pos, q = np.array(pos), np.array(q)
    cp = np.asarray(cpol_bohr)
    E = np.zeros_like(cp)
    for k in range(n_charges):
        d = cp - pos[k]
        r = np.linalg.norm(d, axis=1)
        E += q[k] * d / r[:, None] ** 3
    return E, q, pos
