"""Seeded synthetic packings in LF_DEM's text Configuration_File format.

Sizes follow the reference generator's rules (GenerateInitConfig.cpp:538-573:
bidisperse radii 1 and 1.4 with equal volume (or area) shares, np1 rounded
from the volume share, cubic / square box from the particle volume).
Positions are drawn uniformly at random with a fixed seed and then relaxed by
steepest descent on a harmonic overlap energy until the smallest reduced gap
is above -0.01, the same stopping target as the reference's contact-only
relaxation (GenerateInitConfig.cpp:55-139).  This is an input producer for the
benchmarks and tests, not part of the per-step engine.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass
class Packing:
    position: np.ndarray   # (n, 3) float64
    radius: np.ndarray     # (n,) float64
    lx: float
    ly: float
    lz: float
    np1: int
    np2: int
    vf: float
    le_disp: tuple = (0.0, 0.0)

    @property
    def n(self) -> int:
        return int(self.radius.shape[0])

    @property
    def twodim(self) -> bool:
        return self.ly == 0.0


def box_sizes(n: int, vf: float, a1: float = 1.0, a2: float = 1.4, twodim: bool = False):
    """(np1, np2, lx, ly, lz) by GenerateInitConfig.cpp:538-573 (vf_ratio 0.5)."""
    if twodim:
        pv1, pv2 = math.pi * a1 * a1, math.pi * a2 * a2
    else:
        pv1, pv2 = (4.0 / 3) * math.pi * a1 ** 3, (4.0 / 3) * math.pi * a2 ** 3
    vf1 = vf * 0.5
    vf2 = vf - vf1
    total = n / (vf1 / pv1 + vf2 / pv2)
    np1_tmp = vf1 * total / pv1
    np1 = int(np1_tmp) if np1_tmp - int(np1_tmp) <= 0.5 else int(np1_tmp) + 1
    np2 = n - np1
    pvol = np1 * pv1 + np2 * pv2
    if twodim:
        lz = math.sqrt(pvol / vf)
        return np1, np2, lz, 0.0, lz
    lz = (pvol / vf) ** (1.0 / 3)
    return np1, np2, lz, lz, lz


def _pairs(pos, box, cutoff, twodim):
    from scipy.spatial import cKDTree
    if twodim:
        pts = pos[:, [0, 2]]
        bs = np.array([box[0], box[2]])
    else:
        pts = pos
        bs = np.array(box)
    pts = np.mod(pts, bs)
    pts = np.where(pts >= bs, 0.0, pts)
    tree = cKDTree(pts, boxsize=bs)
    return tree.query_pairs(cutoff, output_type="ndarray")


def generate(n: int, vf: float, seed: int, twodim: bool = False,
             min_gap: float = -0.01, max_iter: int = 20000) -> Packing:
    np1, np2, lx, ly, lz = box_sizes(n, vf, twodim=twodim)
    rng = np.random.default_rng(seed)
    radius = np.concatenate([np.full(np1, 1.0), np.full(np2, 1.4)])
    box = np.array([lx, ly if not twodim else 1.0, lz])
    pos = rng.random((n, 3)) * box
    if twodim:
        pos[:, 1] = 0.0
    amax = radius.max()
    step = 0.25
    for _ in range(max_iter):
        pr = _pairs(pos, (lx, ly if not twodim else 1.0, lz), 2 * amax, twodim)
        if len(pr) == 0:
            break
        i, j = pr[:, 0], pr[:, 1]
        d = pos[j] - pos[i]
        for ax, L in ((0, lx), (2, lz)) + (() if twodim else ((1, ly),)):
            d[:, ax] -= L * np.round(d[:, ax] / L)
        r = np.sqrt((d * d).sum(1))
        ro = radius[i] + radius[j]
        gap = 2 * r / ro - 2
        ov = gap < 0
        if not ov.any() or gap[ov].min() >= min_gap:
            break
        i, j, d, r, ro = i[ov], j[ov], d[ov], r[ov], ro[ov]
        push = (ro - r)[:, None] * d / np.maximum(r, 1e-12)[:, None]
        disp = np.zeros_like(pos)
        np.add.at(disp, i, -0.5 * step * push)
        np.add.at(disp, j, 0.5 * step * push)
        pos += disp
        pos[:, 0] %= lx
        pos[:, 2] %= lz
        if not twodim:
            pos[:, 1] %= ly
    else:
        raise RuntimeError("packing relaxation did not converge")
    # exact [0, L) wrap
    for ax, L in ((0, lx), (2, lz)) + (() if twodim else ((1, ly),)):
        pos[:, ax] = np.mod(pos[:, ax], L)
        pos[pos[:, ax] >= L, ax] = 0.0
    return Packing(position=pos, radius=radius, lx=lx, ly=ly, lz=lz, np1=np1, np2=np2, vf=vf)


def write_conf(p: Packing, path: str) -> None:
    """Text Configuration_File (Configuration.h:287-339)."""
    vf1 = vf2 = p.vf / 2
    with open(path, "w") as f:
        f.write("# np1 np2 vf lx ly lz vf1 vf2 disp\n")
        f.write(f"# {p.np1} {p.np2} {p.vf:.17g} {p.lx:.17g} {p.ly:.17g} {p.lz:.17g} "
                f"{vf1:.17g} {vf2:.17g} 0\n")
        for (x, y, z), a in zip(p.position, p.radius):
            f.write(f"{x:.17g} {y:.17g} {z:.17g} {a:.17g}\n")


def read_conf(path: str) -> Packing:
    """Read a text Configuration_File (Configuration.h:140-172, 313-339)."""
    with open(path) as f:
        h1 = f.readline().split()
        h2 = f.readline().split()
        meta = dict(zip(h1[1:], h2[1:]))
        rows = np.loadtxt(f, ndmin=2)
    pos = rows[:, :3].copy()
    rad = rows[:, 3].copy()
    lx, ly, lz = float(meta["lx"]), float(meta["ly"]), float(meta["lz"])
    disp = (float(meta.get("dispx", 0)), float(meta.get("dispy", 0)))
    np1 = int(meta.get("np1", (rad == rad.min()).sum()))
    np2 = int(meta.get("np2", len(rad) - np1))
    return Packing(position=pos, radius=rad, lx=lx, ly=ly, lz=lz, np1=np1, np2=np2,
                   vf=float(meta.get("vf", 0)), le_disp=disp)
