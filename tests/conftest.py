import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "lammps-lmff_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")
# the reference source tree (present where the fixtures were made, absent on GPU hosts)
REFERENCE = os.environ.get("LMFF_REFERENCE", "/root/reference")
POT = os.path.join(ROOT, "lammps-lmff_gb300", "potentials")
TERSOFF = os.path.join(POT, "BNC.tersoff")
ILP = os.path.join(POT, "BNCH.ILP")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def rel_max(a, b):
    """max |a-b| / max |b|  (max-norm relative error)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.abs(b).max()
    return float(np.abs(a - b).max() / den) if den > 0 else float(np.abs(a - b).max())


def rel_rms(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.sqrt(np.mean(b * b))
    return float(np.sqrt(np.mean((a - b) ** 2)) / den) if den > 0 else 0.0


def min_image(d, lo, hi, periodic):
    d = np.array(d, dtype=np.float64)
    L = np.asarray(hi) - np.asarray(lo)
    for c in range(3):
        if periodic[c]:
            d[..., c] -= L[c] * np.rint(d[..., c] / L[c])
    return d


GOLDEN_SINGLE = ["bilayer_small", "bilayer_small_notaper", "hetero_small", "tiny_images", "edges",
                 "trilayer_alt", "c1_t0", "c1_t100"]
GOLDEN_LISTS = ["bilayer_small", "hetero_small", "tiny_images", "edges", "trilayer_alt"]
# fixtures that carry each style's per-atom virial (vatom_tersoff, vatom_ilp)
GOLDEN_VATOM = ["bilayer_small", "bilayer_small_notaper", "hetero_small", "tiny_images", "edges", "trilayer_alt"]
