"""The LAMMPS package (lammps-lmff_gb300/lammps) inside the reference LAMMPS: an
unchanged input script run with `-sf gb300` must reach the engine through the
reference's own pair_style / pair_coeff parsing.  Needs the reference sources, so it
runs only where they are present; without a GPU the engine reports that there is none."""
import os
import subprocess

import pytest
from conftest import POT, ROOT

from lmff_gb300 import build, capi
from lmff_gb300 import structures as S

REF = os.environ.get("LMFF_REFERENCE", "/root/reference")


@pytest.fixture(scope="module")
def lmp():
    if not os.path.isdir(os.path.join(REF, "Rft")):
        pytest.skip("reference sources not present")
    build.build()
    subprocess.check_call(["make", "-s", "-f", os.path.join(ROOT, "oracle", "ref.mk"), f"REF={REF}", "-j8", "all",
                           "gb300"], cwd=ROOT)
    return os.path.join(ROOT, "oracle", "_ref", "lmp_gb300")


def test_suffix_routes_unchanged_script_to_engine(lmp, tmp_path):
    s = S.displace(S.ab_bilayer_graphene(8, 5), 0.03, seed=2)
    data = tmp_path / "data.lmp"
    S.write_lammps_data(s, str(data))
    script = tmp_path / "in.lmp"
    script.write_text(f"""units metal
atom_style full
boundary p p f
read_data {data}
pair_style hybrid/overlay tersoff ilp/graphene/hbn 16.0 1
pair_coeff * * tersoff {POT}/BNC.tersoff C B N
pair_coeff * * ilp/graphene/hbn {POT}/BNCH.ILP C B N
neighbor 2.0 bin
run 0
""")
    r = subprocess.run([lmp, str(script), str(tmp_path / "out.bin"), "--", "-sf", "gb300", "-log", "none",
                        "-nocite"], capture_output=True, text=True, cwd=str(tmp_path))
    text = r.stdout + r.stderr
    assert "Reading potential file" in text           # the reference's read_file parsed it
    if capi.device_count() == 0:
        assert r.returncode != 0
        assert "tersoff/gb300: no CUDA device" in text  # init_style reached lmff_create
    else:
        assert r.returncode == 0, text


def test_suffix_routes_kolmogorov_crespi_full(lmp, tmp_path):
    """kolmogorov/crespi/full -> kolmogorov/crespi/full/gb300 through the reference's
    own settings / coeff / read_file (12-word CC.KC-full entries)."""
    s = S.displace(S.ab_bilayer_graphene(8, 5), 0.03, seed=3)
    data = tmp_path / "data.lmp"
    S.write_lammps_data(s, str(data), ntypes=1)     # carbon only: every type pair is set
    script = tmp_path / "in.lmp"
    script.write_text(f"""units metal
atom_style full
boundary p p f
read_data {data}
pair_style hybrid/overlay kolmogorov/crespi/full 16.0 1
pair_coeff * * kolmogorov/crespi/full {POT}/CC.KC-full C
pair_modify shift yes
neighbor 2.0 bin
run 0
""")
    r = subprocess.run([lmp, str(script), str(tmp_path / "out.bin"), "--", "-sf", "gb300", "-log", "none",
                        "-nocite"], capture_output=True, text=True, cwd=str(tmp_path))
    text = r.stdout + r.stderr
    if capi.device_count() == 0:
        assert r.returncode != 0
        assert "kolmogorov/crespi/full/gb300: no CUDA device" in text, text
    else:
        assert r.returncode == 0, text
