"""Seeded synthetic polarizable-embedding systems (rigid water boxes).

The reference ships no benchmark inputs, so the benchmark configurations are
generated: rigid waters (O-H 0.9572 A, H-O-H 104.52 deg) at uniformly random
orientations on a jittered cubic lattice filling a cube at 1.0 g/cm^3
(0.03343 waters per A^3); charges O -0.67 / H +0.335; dipoles and traceless
quadrupoles drawn N(0, 0.1) a.u.; isotropic polarizabilities O 5.7 / H 2.3
a.u.; each site excludes its two molecule mates.  The external field comes
from 12 point charges N(0, 0.5) e drawn uniformly in a 3 A sphere about the
box centre (draws closer than 1 A to a site are rejected).

Coordinates are returned in bohr (the potfile reader's AA -> bohr factor
1.8897261246, src/core/potfile_reader.cc:10), and ``write_potfile`` writes the
same system as a ``.pot`` file (AA) for the reference's input path.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

ANG2BOHR = 1.8897261246
WATER_DENSITY = 0.03343  # molecules per A^3 at 1.0 g/cm^3
R_OH = 0.9572
HOH_DEG = 104.52


@dataclass
class WaterBox:
    n_waters: int
    seed: int
    box_aa: float
    xyz: np.ndarray        # (n, 3) bohr, order O H H per molecule
    elements: list
    q: np.ndarray          # (n,)
    mu: np.ndarray         # (n, 3)
    quad: np.ndarray       # (n, 6) traceless
    alpha6: np.ndarray     # (n, 6)
    excl_ptr: np.ndarray   # (n+1,)
    excl_idx: np.ndarray
    charges_xyz: np.ndarray  # (12, 3) bohr
    charges_q: np.ndarray    # (12,)

    @property
    def n(self):
        return self.xyz.shape[0]

    @property
    def alpha_iso(self):
        return (self.alpha6[:, 0] + self.alpha6[:, 3] + self.alpha6[:, 5]) / 3.0

    def external_field(self):
        """E_i = sum_k q_k (r_i - R_k) / |r_i - R_k|^3 (bohr, a.u.)."""
        return point_charge_field(self.xyz, self.charges_xyz, self.charges_q)


def point_charge_field(xyz, cxyz, cq):
    d = xyz[:, None, :] - cxyz[None, :, :]
    r = np.linalg.norm(d, axis=2)
    return (cq[None, :, None] * d / r[:, :, None] ** 3).sum(axis=1).reshape(-1)


def _random_rotations(rng, n):
    # uniform random unit quaternions (Shoemake)
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    a, b = np.sqrt(1 - u1), np.sqrt(u1)
    qx, qy = a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2)
    qz, qw = b * np.sin(2 * np.pi * u3), b * np.cos(2 * np.pi * u3)
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (qy * qy + qz * qz)
    R[:, 0, 1] = 2 * (qx * qy - qz * qw)
    R[:, 0, 2] = 2 * (qx * qz + qy * qw)
    R[:, 1, 0] = 2 * (qx * qy + qz * qw)
    R[:, 1, 1] = 1 - 2 * (qx * qx + qz * qz)
    R[:, 1, 2] = 2 * (qy * qz - qx * qw)
    R[:, 2, 0] = 2 * (qx * qz - qy * qw)
    R[:, 2, 1] = 2 * (qy * qz + qx * qw)
    R[:, 2, 2] = 1 - 2 * (qx * qx + qy * qy)
    return R


def water_box(n_waters: int, seed: int = 0, jitter_aa: float = 0.3,
              n_charges: int = 12) -> WaterBox:
    rng = np.random.default_rng(seed)
    L = (n_waters / WATER_DENSITY) ** (1.0 / 3.0)
    k = int(np.ceil(n_waters ** (1.0 / 3.0)))
    spacing = L / k
    cells = rng.permutation(k ** 3)[:n_waters]
    ijk = np.stack(np.unravel_index(cells, (k, k, k)), axis=1).astype(float)
    O = (ijk + 0.5) * spacing + rng.uniform(-jitter_aa, jitter_aa, size=(n_waters, 3))
    half = np.deg2rad(HOH_DEG) / 2
    h1 = np.array([R_OH * np.sin(half), R_OH * np.cos(half), 0.0])
    h2 = np.array([-R_OH * np.sin(half), R_OH * np.cos(half), 0.0])
    R = _random_rotations(rng, n_waters)
    H1 = O + R @ h1
    H2 = O + R @ h2
    xyz_aa = np.stack([O, H1, H2], axis=1).reshape(-1, 3)
    n = 3 * n_waters
    elements = ["O", "H", "H"] * n_waters
    q = np.tile([-0.67, 0.335, 0.335], n_waters)
    mu = rng.normal(0.0, 0.1, size=(n, 3))
    quad = rng.normal(0.0, 0.1, size=(n, 6))
    tr = (quad[:, 0] + quad[:, 3] + quad[:, 5]) / 3.0
    quad[:, [0, 3, 5]] -= tr[:, None]
    iso = np.tile([5.7, 2.3, 2.3], n_waters)
    alpha6 = np.zeros((n, 6))
    alpha6[:, 0] = alpha6[:, 3] = alpha6[:, 5] = iso
    excl_ptr = np.arange(0, 2 * n + 1, 2, dtype=np.int32)
    base = np.repeat(np.arange(n_waters) * 3, 3)
    mates = np.array([[1, 2], [0, 2], [0, 1]] * n_waters)
    excl_idx = (base[:, None] + mates).reshape(-1).astype(np.int32)
    # point charges within 3 A of the centre, at least 1 A from every site
    centre = np.full(3, L / 2)
    cx, cq = [], []
    while len(cx) < n_charges:
        v = rng.uniform(-3.0, 3.0, size=3)
        if np.linalg.norm(v) > 3.0:
            continue
        c = centre + v
        if np.min(np.linalg.norm(xyz_aa - c, axis=1)) < 1.0:
            continue
        cx.append(c)
        cq.append(rng.normal(0.0, 0.5))
    return WaterBox(n_waters=n_waters, seed=seed, box_aa=L, xyz=xyz_aa * ANG2BOHR,
                    elements=elements, q=q, mu=mu, quad=quad, alpha6=alpha6,
                    excl_ptr=excl_ptr, excl_idx=excl_idx,
                    charges_xyz=np.array(cx) * ANG2BOHR, charges_q=np.array(cq))


def write_potfile(box: WaterBox, path: str):
    """Writes the box as a .pot file in AA (read back, positions round-trip to
    ~1e-10 bohr)."""
    n = box.n
    xyz_aa = box.xyz / ANG2BOHR
    with open(path, "w") as f:
        f.write("! synthetic water box, seed %d\n@COORDINATES\n%d\nAA\n" % (box.seed, n))
        for i in range(n):
            f.write("%s %.12f %.12f %.12f %d\n" % (box.elements[i], *xyz_aa[i], i + 1))
        f.write("@MULTIPOLES\nORDER 0\n%d\n" % n)
        for i in range(n):
            f.write("%d %.12f\n" % (i + 1, box.q[i]))
        f.write("ORDER 1\n%d\n" % n)
        for i in range(n):
            f.write("%d %.12f %.12f %.12f\n" % (i + 1, *box.mu[i]))
        f.write("ORDER 2\n%d\n" % n)
        for i in range(n):
            f.write("%d %.12f %.12f %.12f %.12f %.12f %.12f\n" % (i + 1, *box.quad[i]))
        f.write("@POLARIZABILITIES\nORDER 1 1\n%d\n" % n)
        for i in range(n):
            f.write("%d %.12f %.12f %.12f %.12f %.12f %.12f\n" % (i + 1, *box.alpha6[i]))
        f.write("EXCLISTS\n%d 3\n" % n)
        for i in range(n):
            e = box.excl_idx[box.excl_ptr[i]:box.excl_ptr[i + 1]]
            f.write("%d %d %d\n" % (i + 1, e[0] + 1, e[1] + 1))


def snapshot_sizes(n_snapshots: int = 256, seed: int = 1000, lo: int = 500, hi: int = 20000):
    """Site counts of the batched configuration: 3 * round(exp U[ln(lo/3), ln(hi/3)])."""
    rng = np.random.default_rng(seed)
    nw = np.round(np.exp(rng.uniform(np.log(lo / 3), np.log(hi / 3), size=n_snapshots)))
    return (3 * nw).astype(int)
