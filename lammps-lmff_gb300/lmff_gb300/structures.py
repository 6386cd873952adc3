"""Seeded generators for the layered systems the engine is measured and tested on.

Atom types follow one fixed convention everywhere in this package: 1 = C, 2 = B, 3 = N,
matching ``pair_coeff * * tersoff BNC.tersoff C B N`` and
``pair_coeff * * ilp/graphene/hbn BNCH.ILP C B N``.  Molecule ids mark layers, as the
ILP style requires (``pair_ilp_graphene_hbn.cpp:504,597`` interacts only
``molecule[i] != molecule[j]``; ``:732`` builds the intralayer list from
``molecule[i] == molecule[j]``).

Honeycomb layers are built on the rectangular 4-atom cell a = sqrt(3)*d, b = 3*d with
basis (0,0), (a/2, d/2), (a/2, 3d/2), (0, 2d), d the bond length.  Twisted layers are made
commensurate with the rectangular periodic box by a small homogeneous strain, which every
generator reports in ``meta`` (no exactly commensurate cell exists for an arbitrary twist
or for the 2% graphene/hBN lattice mismatch).
"""
from __future__ import annotations

import dataclasses
import math
import os
from typing import Dict, List, Optional

import numpy as np

A_CC_GRAPHENE = 1.42
A_CC_HBN = 1.45
MASSES = {1: 12.011, 2: 10.811, 3: 14.0067}
BOLTZ_METAL = 8.617343e-5          # eV/K        (LAMMPS update.cpp, units metal)
MVV2E_METAL = 1.0364269e-4         # amu*A^2/ps^2 -> eV


@dataclasses.dataclass
class System:
    x: np.ndarray                  # (N,3) float64, Angstrom
    type: np.ndarray               # (N,)  int32, 1=C 2=B 3=N
    mol: np.ndarray                # (N,)  int64 layer id
    tag: np.ndarray                # (N,)  int64, 1..N
    box_lo: np.ndarray             # (3,)
    box_hi: np.ndarray             # (3,)
    periodic: np.ndarray           # (3,) bool
    v: Optional[np.ndarray] = None  # (N,3) Angstrom/ps
    meta: Dict = dataclasses.field(default_factory=dict)
    # LAMMPS tilt factors (xy, xz, yz) of a triclinic box, None for an orthogonal one:
    # the box edges are (hi-lo)_x (1,0,0), (xy, (hi-lo)_y, 0), (xz, yz, (hi-lo)_z)
    tilt: Optional[np.ndarray] = None

    @property
    def n(self) -> int:
        return int(self.x.shape[0])

    def type_masses(self) -> np.ndarray:
        """Mass of each type (index t-1): a data file's Masses section, else the 1=C,
        2=B, 3=N convention."""
        if "type_masses" in self.meta:
            return np.asarray(self.meta["type_masses"], dtype=np.float64)
        return np.array([MASSES[t] for t in range(1, 4)])

    def masses(self) -> np.ndarray:
        return self.type_masses()[self.type - 1]

    def copy(self) -> "System":
        return System(self.x.copy(), self.type.copy(), self.mol.copy(), self.tag.copy(),
                      self.box_lo.copy(), self.box_hi.copy(), self.periodic.copy(),
                      None if self.v is None else self.v.copy(), dict(self.meta),
                      None if self.tilt is None else self.tilt.copy())


# --------------------------------------------------------------------------- layers

def _rect_layer(nx: int, ny: int, a_cc: float, species=(1, 1)) -> np.ndarray:
    """Unrotated honeycomb layer on nx x ny rectangular cells; returns (N,4) [x,y,0,type]."""
    a = math.sqrt(3.0) * a_cc
    d = a_cc
    basis = [(0.0, 0.0, species[0]), (a / 2, d / 2, species[1]),
             (a / 2, 1.5 * d, species[0]), (0.0, 2.0 * d, species[1])]
    out = []
    for iy in range(ny):
        for ix in range(nx):
            for bx, by, t in basis:
                out.append((ix * a + bx, iy * 3 * d + by, 0.0, t))
    return np.array(out, dtype=np.float64)


def _commensurate_layer(lx: float, ly: float, a_cc: float, theta_deg: float,
                        species=(1, 1), shift=(0.0, 0.0)):
    """Honeycomb layer rotated by theta, strained to tile the box [0,lx) x [0,ly).

    Returns (atoms (N,4), strain_max) where strain_max is the largest principal
    strain of the homogeneous deformation that makes the layer commensurate.
    """
    a = math.sqrt(3.0) * a_cc
    th = math.radians(theta_deg)
    rot = np.array([[math.cos(th), -math.sin(th)], [math.sin(th), math.cos(th)]])
    a1 = rot @ np.array([a, 0.0])
    a2 = rot @ np.array([a / 2, a * math.sqrt(3.0) / 2])
    lat = np.stack([a1, a2], axis=1)
    s1 = np.rint(np.linalg.solve(lat, [lx, 0.0])).astype(np.int64)
    s2 = np.rint(np.linalg.solve(lat, [0.0, ly])).astype(np.int64)
    t1 = lat @ s1
    t2 = lat @ s2
    fdef = np.array([[lx, 0.0], [0.0, ly]]) @ np.linalg.inv(np.stack([t1, t2], axis=1))
    strain = 0.5 * (fdef.T @ fdef - np.eye(2))
    strain_max = float(np.max(np.abs(np.linalg.eigvalsh(strain))))
    p1, q1 = int(s1[0]), int(s1[1])
    p2, q2 = int(s2[0]), int(s2[1])
    det = p1 * q2 - q1 * p2
    if det == 0:
        raise ValueError("degenerate commensurate cell")
    corners = np.array([[0, 0], [p1, q1], [p2, q2], [p1 + p2, q1 + q2]])
    mlo, nlo = corners.min(axis=0) - 1
    mhi, nhi = corners.max(axis=0) + 1
    mm, nn = np.meshgrid(np.arange(mlo, mhi + 1), np.arange(nlo, nhi + 1), indexing="ij")
    mm = mm.ravel()
    nn = nn.ravel()
    # fractional coordinates in the supercell basis, exact in integers: f = S^-1 (m,n)
    f1n = mm * q2 - nn * p2
    f2n = -mm * q1 + nn * p1
    if det < 0:
        f1n, f2n, det = -f1n, -f2n, -det
    keep = (f1n >= 0) & (f1n < det) & (f2n >= 0) & (f2n < det)
    f1 = f1n[keep] / det
    f2 = f2n[keep] / det
    base = np.stack([f1 * lx, f2 * ly], axis=1)
    delta = fdef @ (rot @ np.array([a / 2, a_cc / 2]))
    sh = np.asarray(shift, dtype=np.float64)
    pts = []
    for off, t in ((np.zeros(2), species[0]), (delta, species[1])):
        p = base + off + sh
        p[:, 0] = np.mod(p[:, 0], lx)
        p[:, 1] = np.mod(p[:, 1], ly)
        pts.append(np.column_stack([p, np.zeros(len(p)), np.full(len(p), t)]))
    atoms = np.concatenate(pts, axis=0)
    return atoms, strain_max


def _assemble(layers: List[np.ndarray], zs: List[float], mols: List[int], lx: float, ly: float,
              vacuum: float, periodic_z: bool = False, meta: Optional[Dict] = None) -> System:
    xs, ts, ms = [], [], []
    for atoms, z, m in zip(layers, zs, mols):
        p = atoms[:, :3].copy()
        p[:, 2] = z
        xs.append(p)
        ts.append(atoms[:, 3].astype(np.int32))
        ms.append(np.full(len(atoms), m, dtype=np.int64))
    x = np.concatenate(xs)
    t = np.concatenate(ts)
    mol = np.concatenate(ms)
    zlo = min(zs) - vacuum / 2
    zhi = max(zs) + vacuum / 2
    box_lo = np.array([0.0, 0.0, zlo])
    box_hi = np.array([lx, ly, zhi])
    per = np.array([True, True, periodic_z])
    tag = np.arange(1, len(x) + 1, dtype=np.int64)
    return System(x, t, mol, tag, box_lo, box_hi, per, None, dict(meta or {}))


def ab_bilayer_graphene(nx: int = 30, ny: int = 30, spacing: float = 3.4,
                        vacuum: float = 30.0) -> System:
    """AB-stacked bilayer graphene, C-C 1.42 A, on nx x ny rectangular 4-atom cells.

    nx = ny = 30 gives the 7,200-atom plain-FP64 parity workload (box 73.79 x 127.80 A,
    layers at z = 0 and 3.4, 30 A of z vacuum, periodic x/y)."""
    a = math.sqrt(3.0) * A_CC_GRAPHENE
    lx, ly = nx * a, ny * 3 * A_CC_GRAPHENE
    l1 = _rect_layer(nx, ny, A_CC_GRAPHENE)
    l2 = l1.copy()
    l2[:, 1] = np.mod(l2[:, 1] + A_CC_GRAPHENE, ly)
    return _assemble([l1, l2], [0.0, spacing], [1, 2], lx, ly, vacuum,
                     meta={"kind": "ab_bilayer_graphene", "nx": nx, "ny": ny, "spacing": spacing})


def graphite_slab(nlayers: int = 10, nx: int = 342, ny: int = 197, spacing: float = 3.35,
                  mol_mode: str = "alternate", vacuum: float = 30.0) -> System:
    """AB-stacked graphite slab, periodic x/y.

    Defaults give the 10-layer, 2.7M-atom slab (269,496 atoms per layer, box
    841.2 x 839.2 A, 3.35 A spacing).  mol_mode "alternate" gives layers molecule ids
    1,2,1,2,... (only odd layer separations interact through ILP); "unique" gives each
    layer its own id."""
    a = math.sqrt(3.0) * A_CC_GRAPHENE
    lx, ly = nx * a, ny * 3 * A_CC_GRAPHENE
    base = _rect_layer(nx, ny, A_CC_GRAPHENE)
    layers, zs, mols = [], [], []
    for k in range(nlayers):
        l = base.copy()
        if k % 2 == 1:
            l[:, 1] = np.mod(l[:, 1] + A_CC_GRAPHENE, ly)
        layers.append(l)
        zs.append(k * spacing)
        mols.append(1 + (k % 2) if mol_mode == "alternate" else k + 1)
    return _assemble(layers, zs, mols, lx, ly, vacuum,
                     meta={"kind": "graphite_slab", "nlayers": nlayers, "nx": nx, "ny": ny,
                           "spacing": spacing, "mol_mode": mol_mode})


def twisted_bilayer(nx: int, ny: int, theta_deg: float, top: str = "hbn", spacing: float = 3.4,
                    shift=(0.0, 0.0), vacuum: float = 30.0) -> System:
    """Graphene (bottom, unstrained, nx x ny rectangular cells) under a top layer
    ("graphene" or "hbn") twisted by theta and strained to be commensurate with the box.
    meta["strain_max"] is the top layer's largest principal strain."""
    a = math.sqrt(3.0) * A_CC_GRAPHENE
    lx, ly = nx * a, ny * 3 * A_CC_GRAPHENE
    bottom = _rect_layer(nx, ny, A_CC_GRAPHENE)
    if top == "hbn":
        upper, strain = _commensurate_layer(lx, ly, A_CC_HBN, theta_deg, species=(2, 3), shift=shift)
    else:
        upper, strain = _commensurate_layer(lx, ly, A_CC_GRAPHENE, theta_deg, species=(1, 1),
                                            shift=shift)
    return _assemble([bottom, upper], [0.0, spacing], [1, 2], lx, ly, vacuum,
                     meta={"kind": "twisted_bilayer", "top": top, "theta_deg": theta_deg,
                           "strain_max": strain, "nx": nx, "ny": ny, "spacing": spacing})


def twisted_graphene_hbn_500k(seed: int = 2, theta_deg: float = 0.6) -> System:
    """Twisted graphene/hBN, 0.6 degrees, about 500k atoms over two layers, with the
    per-atom N(0, 0.02 A) displacement applied from ``seed``."""
    s = twisted_bilayer(329, 190, theta_deg, top="hbn", spacing=3.4)
    rng = np.random.default_rng(seed)
    s.x += rng.normal(0.0, 0.02, size=s.x.shape)
    s.meta["displacement_sigma"] = 0.02
    return s


def hex_layers(m: int, n: int, nlayers: int = 2, spacing: float = 3.4, species: str = "C",
               mol_mode: str = "unique", periodic_z: bool = False, xz: float = 0.0, yz: float = 0.0,
               vacuum: float = 30.0) -> System:
    """AB-stacked honeycomb layers in a triclinic (hexagonal) cell of m x n primitive
    cells, C-C 1.42 A: in-plane edges m a (1, 0) and n a (1/2, sqrt(3)/2), a = sqrt(3) d,
    so LAMMPS's tilt xy = n a / 2 (n < m keeps it below half the x edge, LAMMPS's skew
    limit).  Primitive-cell basis (0, 0) and (a1 + a2)/3; odd layers shifted by
    (a1 + a2)/3.  species "C" or "BN" (odd layers B/N on the same lattice: strained
    hBN, a test geometry).  periodic_z: the z edge is (xz, yz, nlayers * spacing) and
    the stacking continues through it (each layer also slides by its height fraction of
    (xz, yz)); otherwise z is not periodic, with ``vacuum`` A around the layers.
    mol_mode "unique" (layer k has id k+1) or "alternate" (1, 2, 1, 2, ...)."""
    a = math.sqrt(3.0) * A_CC_GRAPHENE
    lx, ly, xy = m * a, n * a * math.sqrt(3.0) / 2.0, n * a / 2.0
    if periodic_z:
        zlo, lz = -spacing / 2.0, nlayers * spacing
    else:
        xz = yz = 0.0
        zlo, lz = -vacuum / 2.0, (nlayers - 1) * spacing + vacuum
    h = np.array([[lx, xy, xz], [0.0, ly, yz], [0.0, 0.0, lz]])
    lo = np.array([0.0, 0.0, zlo])
    xs, ts, ms = [], [], []
    ii, jj = np.meshgrid(np.arange(m), np.arange(n), indexing="ij")
    ii, jj = ii.ravel().astype(float), jj.ravel().astype(float)
    for k in range(nlayers):
        f0 = (k % 2) / 3.0
        for b, f in enumerate((f0, f0 + 1.0 / 3.0)):
            lam = np.stack([(ii + f) / m, (jj + f) / n, np.full(ii.shape, (k * spacing - zlo) / lz)], axis=1)
            xs.append(lo + lam @ h.T)
            t = 1 if species == "C" or k % 2 == 0 else 2 + b
            ts.append(np.full(len(ii), t, dtype=np.int32))
            ms.append(np.full(len(ii), (k + 1) if mol_mode == "unique" else 1 + k % 2, dtype=np.int64))
    x = np.concatenate(xs)
    tag = np.arange(1, len(x) + 1, dtype=np.int64)
    return System(x, np.concatenate(ts), np.concatenate(ms), tag, lo, lo + np.array([lx, ly, lz]),
                  np.array([True, True, periodic_z]), None,
                  {"kind": "hex_layers", "m": m, "n": n, "nlayers": nlayers, "spacing": spacing},
                  np.array([xy, xz, yz]))


def flake_edges(nx: int = 4, ny: int = 3) -> System:
    """Bilayer ribbon periodic in x only, plus one isolated and one dangling atom in each
    layer: exercises atoms with 0, 1, 2 and 3 intralayer neighbours (normal cases
    nilp <= 1, 2, 3)."""
    a = math.sqrt(3.0) * A_CC_GRAPHENE
    lx = nx * a
    l1 = _rect_layer(nx, ny, A_CC_GRAPHENE)
    l2 = l1.copy()
    l2[:, 1] += A_CC_GRAPHENE
    ly_span = ny * 3 * A_CC_GRAPHENE
    iso1 = np.array([[lx / 2, ly_span + 4.0, 0.0, 1.0],          # no neighbour
                     [0.0, -A_CC_GRAPHENE, 0.0, 1.0]])            # dangling: one neighbour
    iso2 = np.array([[lx / 2, ly_span + 4.0 + A_CC_GRAPHENE, 0.0, 1.0],
                     [0.0, 0.0, 0.0, 1.0]])
    l1 = np.concatenate([l1, iso1])
    l2 = np.concatenate([l2, iso2])
    s = _assemble([l1, l2], [0.0, 3.4], [1, 2], lx, 1.0, 30.0)
    s.box_lo[1] = -10.0
    s.box_hi[1] = ly_span + 16.0
    s.periodic = np.array([True, False, False])
    s.meta = {"kind": "flake_edges", "nx": nx, "ny": ny}
    return s


# ------------------------------------------------------------------ perturbations

def displace(s: System, sigma: float, seed: int) -> System:
    out = s.copy()
    rng = np.random.default_rng(seed)
    out.x = out.x + rng.normal(0.0, sigma, size=out.x.shape)
    out.meta["displacement_sigma"] = sigma
    return out


def thermalize(s: System, temp: float, seed: int) -> System:
    """Gaussian velocities at ``temp`` (K): zero total momentum, then scaled so the
    kinetic temperature (3N-3 degrees of freedom) is exactly ``temp``."""
    out = s.copy()
    rng = np.random.default_rng(seed)
    m = out.masses()
    v = rng.normal(0.0, 1.0, size=out.x.shape) / np.sqrt(m)[:, None]
    v -= (m[:, None] * v).sum(axis=0) / m.sum()
    ke = 0.5 * MVV2E_METAL * float((m[:, None] * v * v).sum())
    dof = 3 * out.n - 3
    t_now = 2.0 * ke / (dof * BOLTZ_METAL)
    out.v = v * math.sqrt(temp / t_now)
    out.meta["temperature"] = temp
    return out


def wrap(s: System) -> System:
    out = s.copy()
    L = out.box_hi - out.box_lo
    for c in range(3):
        if out.periodic[c]:
            out.x[:, c] = out.box_lo[c] + np.mod(out.x[:, c] - out.box_lo[c], L[c])
    return out


# -------------------------------------------------------------------- replica sets

def _rect_for_count(n_layer: int, a_cc: float = A_CC_GRAPHENE):
    a = math.sqrt(3.0) * a_cc
    b = 3 * a_cc
    cells = max(1, round(n_layer / 4))
    nx = max(1, round(math.sqrt(cells * b / a)))
    ny = max(1, round(cells / nx))
    return nx, ny


def replica_set(count: int = 256, nmin: int = 500, nmax: int = 20000, seed: int = 4) -> List[System]:
    """Independent bilayer replicas: 50/50 graphene/graphene and graphene/hBN, total atom
    counts log-uniform in [nmin, nmax], twist U[0,5] degrees, lateral shift uniform in one
    unit cell, interlayer spacing U[3.2,3.6] A.  Every periodic side is at least 20 A."""
    rng = np.random.default_rng(seed)
    out = []
    for r in range(count):
        ntot = math.exp(rng.uniform(math.log(nmin), math.log(nmax)))
        top = "graphene" if r % 2 == 0 else "hbn"
        theta = float(rng.uniform(0.0, 5.0))
        spacing = float(rng.uniform(3.2, 3.6))
        a = math.sqrt(3.0) * A_CC_GRAPHENE
        shift = (float(rng.uniform(0, a)), float(rng.uniform(0, 3 * A_CC_GRAPHENE)))
        nx, ny = _rect_for_count(int(ntot / 2))
        nx = max(nx, math.ceil(20.0 / a))
        ny = max(ny, math.ceil(20.0 / (3 * A_CC_GRAPHENE)))
        best = None
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                cx, cy = nx + dx, ny + dy
                if cx * a < 20.0 or cy * 3 * A_CC_GRAPHENE < 20.0:
                    continue
                s = twisted_bilayer(cx, cy, theta, top=top, spacing=spacing, shift=shift)
                if best is None or s.meta["strain_max"] < best.meta["strain_max"]:
                    best = s
        best.meta["replica"] = r
        out.append(best)
    return out


# ----------------------------------------------------------------- replicate

def replicate(s: System, nx: int, ny: int, nz: int) -> System:
    """LAMMPS ``replicate nx ny nz`` on an orthogonal box (replicate.cpp): the box grows
    to n times each length from the same lower corner; copy (ix, iy, iz) of an atom is
    shifted by (ix Lx, iy Ly, iz Lz), wrapped into the new box on periodic dimensions
    (Domain::remap), and gets tag + k*maxtag and, when its molecule id is positive,
    mol + k*maxmol, with k = iz*ny*nx + iy*nx + ix.  Copies are appended in the loop
    order ix, iy, iz (outer to inner) and atoms in their order within each copy.
    Note the molecule offset: a layer replicated in-plane becomes several molecules, as
    in the reference, which the ILP style then treats as different layers."""
    if min(nx, ny, nz) < 1:
        raise ValueError("replicate counts must be >= 1")
    L = s.box_hi - s.box_lo
    maxtag = int(s.tag.max()) if s.n else 0
    maxmol = int(s.mol.max()) if s.n else 0
    new_hi = s.box_lo + L * np.array([nx, ny, nz])
    xs, ts, ms, gs, vs = [], [], [], [], []
    for ix in range(nx):
        for iy in range(ny):
            for iz in range(nz):
                k = iz * ny * nx + iy * nx + ix
                x = s.x + L * np.array([ix, iy, iz])
                for c in range(3):
                    if s.periodic[c]:
                        Lc = new_hi[c] - s.box_lo[c]
                        x[:, c] = s.box_lo[c] + np.mod(x[:, c] - s.box_lo[c], Lc)
                xs.append(x)
                ts.append(s.type.copy())
                ms.append(np.where(s.mol > 0, s.mol + k * maxmol, s.mol))
                gs.append(s.tag + k * maxtag)
                if s.v is not None:
                    vs.append(s.v.copy())
    meta = dict(s.meta)
    meta["replicate"] = (nx, ny, nz)
    return System(np.concatenate(xs), np.concatenate(ts).astype(np.int32), np.concatenate(ms).astype(np.int64),
                  np.concatenate(gs).astype(np.int64), s.box_lo.copy(), new_hi, s.periodic.copy(),
                  np.concatenate(vs) if vs else None, meta)


# ------------------------------------------------------------------------- input

_HEADER_KEYS = {"atoms", "bonds", "angles", "dihedrals", "impropers", "atom types", "bond types", "angle types",
                "dihedral types", "improper types", "extra bond per atom", "extra angle per atom",
                "extra dihedral per atom", "extra improper per atom", "extra special per atom", "ellipsoids",
                "lines", "triangles", "bodies"}
_SECTIONS = {"Atoms", "Velocities", "Masses", "Bonds", "Angles", "Dihedrals", "Impropers", "Pair Coeffs",
             "PairIJ Coeffs", "Bond Coeffs", "Angle Coeffs", "Dihedral Coeffs", "Improper Coeffs",
             "BondBond Coeffs", "BondAngle Coeffs", "MiddleBondTorsion Coeffs", "EndBondTorsion Coeffs",
             "AngleTorsion Coeffs", "AngleAngleTorsion Coeffs", "BondBond13 Coeffs", "AngleAngle Coeffs",
             "Ellipsoids", "Lines", "Triangles", "Bodies"}


def read_lammps_data(path: str, periodic=(True, True, True)) -> System:
    """A LAMMPS data file in atom_style full (read_data, read_data.cpp): header counts
    and box, then sections.  Atoms lines are ``id mol type q x y z [ix iy iz]``
    (coordinates kept as written, image flags kept in meta["image"]); Masses and
    Velocities are read; other sections are skipped by their header counts.  Atoms are
    returned in file order; a tilted box's ``xy xz yz`` go to ``tilt``.  ``periodic`` is
    the input script's ``boundary`` (a data file does not carry it)."""
    lines = open(path).read().split("\n")
    counts: Dict[str, int] = {}
    lo = np.zeros(3)
    hi = np.zeros(3)
    tilt = None
    k = 1                                     # line 1 is a title
    while k < len(lines):
        raw = lines[k].split("#", 1)[0].strip()
        if not raw:
            k += 1
            continue
        if raw in _SECTIONS or raw.split()[0] in _SECTIONS:
            break
        w = raw.split()
        if len(w) >= 4 and w[-2:] in (["xlo", "xhi"], ["ylo", "yhi"], ["zlo", "zhi"]):
            c = "xyz".index(w[-2][0])
            lo[c], hi[c] = float(w[0]), float(w[1])
        elif len(w) >= 6 and w[-3:] == ["xy", "xz", "yz"]:
            tilt = np.array([float(t) for t in w[:3]])
        else:
            key = " ".join(w[1:])
            if key not in _HEADER_KEYS:
                raise ValueError(f"{path}:{k + 1}: unknown header line '{raw}'")
            counts[key] = int(w[0])
        k += 1
    natoms = counts.get("atoms", 0)
    ntypes = counts.get("atom types", 0)
    x = np.zeros((natoms, 3))
    typ = np.zeros(natoms, dtype=np.int32)
    mol = np.zeros(natoms, dtype=np.int64)
    tag = np.zeros(natoms, dtype=np.int64)
    img = np.zeros((natoms, 3), dtype=np.int64)
    v = None
    tmass = np.zeros(ntypes)
    have_atoms = False
    section_len = {"Atoms": natoms, "Velocities": natoms, "Masses": ntypes, "Bonds": counts.get("bonds", 0),
                   "Angles": counts.get("angles", 0), "Dihedrals": counts.get("dihedrals", 0),
                   "Impropers": counts.get("impropers", 0)}
    coeff_len = {"Bond Coeffs": "bond types", "Angle Coeffs": "angle types", "Dihedral Coeffs": "dihedral types",
                 "Improper Coeffs": "improper types"}

    def body(start, n):
        out, j = [], start
        while len(out) < n:
            if j >= len(lines):
                raise ValueError(f"{path}: section ended after {len(out)} of {n} lines")
            t = lines[j].split("#", 1)[0].strip()
            if t:
                out.append(t.split())
            j += 1
        return out, j

    while k < len(lines):
        raw = lines[k].split("#", 1)[0].strip()
        if not raw:
            k += 1
            continue
        name = raw
        if name not in _SECTIONS:
            raise ValueError(f"{path}:{k + 1}: unknown section '{raw}'")
        if name in section_len:
            n = section_len[name]
        elif name in coeff_len:
            n = counts.get(coeff_len[name], 0)
        elif name in ("Pair Coeffs",):
            n = ntypes
        elif name == "PairIJ Coeffs":
            n = ntypes * (ntypes + 1) // 2
        else:
            raise ValueError(f"{path}: section '{name}' is not supported")
        rows, k = body(k + 1, n)
        if name == "Atoms":
            have_atoms = True
            for r, w in enumerate(rows):
                if len(w) not in (7, 10):
                    raise ValueError(f"{path}: Atoms line '{' '.join(w)}' is not atom_style full")
                tag[r], mol[r], typ[r] = int(w[0]), int(w[1]), int(w[2])
                x[r] = [float(w[4]), float(w[5]), float(w[6])]
                if len(w) == 10:
                    img[r] = [int(w[7]), int(w[8]), int(w[9])]
        elif name == "Masses":
            for w in rows:
                tmass[int(w[0]) - 1] = float(w[1])
        elif name == "Velocities":
            if not have_atoms:
                raise ValueError(f"{path}: Velocities before Atoms")
            index = {int(t): r for r, t in enumerate(tag)}
            v = np.zeros((natoms, 3))
            for w in rows:
                v[index[int(w[0])]] = [float(w[1]), float(w[2]), float(w[3])]
    if not have_atoms:
        raise ValueError(f"{path}: no Atoms section")
    if typ.size and (typ.min() < 1 or typ.max() > ntypes):
        raise ValueError(f"{path}: atom type outside 1..{ntypes}")
    meta = {"kind": "data_file", "path": os.path.basename(path), "ntypes": ntypes, "image": img}
    if np.all(tmass > 0):
        meta["type_masses"] = tmass
    return System(x, typ, mol, tag, lo, hi, np.array(periodic, dtype=bool), v, meta, tilt)


# ------------------------------------------------------------------------- output

def write_lammps_data(s: System, path: str, ntypes: int = 3) -> None:
    """LAMMPS data file, atom_style full (id mol type q x y z), with Velocities if set."""
    with open(path, "w") as fh:
        fh.write("LAMMPS data file written by lmff_gb300.structures\n\n")
        fh.write(f"{s.n} atoms\n{ntypes} atom types\n\n")
        for c, nm in enumerate("xyz"):
            fh.write(f"{s.box_lo[c]:.17g} {s.box_hi[c]:.17g} {nm}lo {nm}hi\n")
        if s.tilt is not None:
            fh.write(f"{s.tilt[0]:.17g} {s.tilt[1]:.17g} {s.tilt[2]:.17g} xy xz yz\n")
        fh.write("\nMasses\n\n")
        for t in range(1, ntypes + 1):
            fh.write(f"{t} {MASSES[t]}\n")
        fh.write("\nAtoms # full\n\n")
        for i in range(s.n):
            fh.write(f"{int(s.tag[i])} {int(s.mol[i])} {int(s.type[i])} 0.0 "
                     f"{s.x[i,0]:.17g} {s.x[i,1]:.17g} {s.x[i,2]:.17g}\n")
        if s.v is not None:
            fh.write("\nVelocities\n\n")
            for i in range(s.n):
                fh.write(f"{int(s.tag[i])} {s.v[i,0]:.17g} {s.v[i,1]:.17g} {s.v[i,2]:.17g}\n")
