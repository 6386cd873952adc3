"""Generate the golden fixtures in tests/golden/ by running the REFERENCE implementation.

The reference snapshot ships no tests and no reference outputs, so the fixtures are made
here: each case's structure comes from lmff_gb300.structures (seeded), is written as a
LAMMPS data file, and is run through the reference's own pair styles
(pair_style hybrid/overlay tersoff ilp/graphene/hbn, unchanged BNC.tersoff / BNCH.ILP)
by the harness that oracle/ref.mk builds from the reference sources
(oracle/_ref/lmff_ref).  Needs the reference checkout, so it runs only in a container
that has it:

    make -f oracle/ref.mk REF=/root/reference -j8
    python tests/golden/make_golden.py

Every fixture stores the inputs (x, v, type, mol, tag, box, periodicity, potential
settings) and the reference outputs (forces, per-style energies, ILP pvector, fdotr
virial, per-atom energy, each sub-style's per-atom virial as its tallies leave it, in
LAMMPS order xx yy zz xy xz yz; for list cases the full Verlet list and the ILP intralayer list
as (tag_i, tag_j, image) triples with image = sum_c ((s_c+8)&15) << 4c).
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "lammps-lmff_gb300"))
from lmff_gb300 import structures as S  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "lmff_ref")
POT = os.path.join(ROOT, "lammps-lmff_gb300", "potentials")
OUT = os.path.dirname(os.path.abspath(__file__))


def read_records(path):
    out = {}
    data = open(path, "rb").read()
    off = 0
    while off < len(data):
        name = data[off:off + 16].split(b"\0")[0].decode()
        off += 16
        kind = chr(data[off])
        off += 1
        n = int(np.frombuffer(data[off:off + 8], dtype=np.int64)[0])
        off += 8
        dt = np.float64 if kind == "d" else np.int64
        out[name] = np.frombuffer(data[off:off + 8 * n], dtype=dt).copy()
        off += 8 * n
    return out


def run_reference(s: S.System, tap_flag=1, nsteps=0, dt=0.001, lists=False, cut=16.0, interlayer="ilp"):
    """interlayer "ilp": ilp/graphene/hbn with BNCH.ILP; "kc": kolmogorov/crespi/full
    with CC.KC-full (carbon only: types B and N are NULL for it)."""
    if interlayer == "kc":
        inter = (f"pair_style hybrid/overlay tersoff kolmogorov/crespi/full {cut} {tap_flag}\n"
                 f"pair_coeff * * tersoff {POT}/BNC.tersoff C B N\n"
                 f"pair_coeff * * kolmogorov/crespi/full {POT}/CC.KC-full C NULL NULL\n"
                 f"pair_modify shift yes")
    else:
        inter = (f"pair_style hybrid/overlay tersoff ilp/graphene/hbn {cut} {tap_flag}\n"
                 f"pair_coeff * * tersoff {POT}/BNC.tersoff C B N\n"
                 f"pair_coeff * * ilp/graphene/hbn {POT}/BNCH.ILP C B N")
    with tempfile.TemporaryDirectory() as td:
        data = os.path.join(td, "data.lmp")
        S.write_lammps_data(s, data)
        bnd = " ".join("p" if p else "f" for p in s.periodic)
        script = f"""units metal
atom_style full
boundary {bnd}
atom_modify map array
read_data {data}
{inter}
neighbor 2.0 bin
neigh_modify every 1 delay 0 check yes one 10000 page 200000
compute peatom all pe/atom pair
compute pesum all reduce sum c_peatom
compute satom all stress/atom NULL pair
compute vsum all reduce sum c_satom[1]
thermo_style custom step pe c_pesum press c_vsum
thermo {max(nsteps, 1)}
timestep {dt}
"""
        if nsteps:
            script += "fix 1 all nve\n"
        script += f"run {nsteps}\n"
        inp = os.path.join(td, "in.lmp")
        open(inp, "w").write(script)
        out = os.path.join(td, "out.bin")
        args = [HARNESS, inp, out] + (["lists"] if lists else [])
        subprocess.check_call(args)
        return read_records(out)


REF = os.environ.get("LMFF_REFERENCE", "/root/reference")
CASE = os.path.join(REF, "Cases", "case_5016")
# the pair setup of the reference's own case script (Cases/case_5016/in.replicate.ilp_tersoff:77-81)
CASE_PAIR = f"""pair_style hybrid/overlay tersoff ilp/graphene/hbn 16.0 0
pair_coeff * * tersoff {POT}/C.opt.tersoff NULL C(O) C(O) C(O) C(O) C(O)
pair_coeff * * ilp/graphene/hbn {POT}/BNCH.ILP C C C C C C
"""


def run_case(extra_setup="", run="run 0", flags=()):
    """The reference's case_5016 data file through the reference: read_data, the
    case's pair setup, then `extra_setup` and `run`."""
    with tempfile.TemporaryDirectory() as td:
        script = f"""units metal
atom_style full
boundary p p p
atom_modify map array
read_data {CASE}/inf0.data
{extra_setup}
{CASE_PAIR}
neighbor 2.0 bin
neigh_modify every 1 delay 0 check yes one 20000 page 200000
compute peatom all pe/atom pair
compute pesum all reduce sum c_peatom
thermo_style custom step pe c_pesum press
{run}
"""
        inp = os.path.join(td, "in.lmp")
        open(inp, "w").write(script)
        out = os.path.join(td, "out.bin")
        subprocess.check_call([HARNESS, inp, out, *flags])
        return read_records(out)


def pack_case(r, extra=None):
    n = len(r["tag"])
    d = {"x": r["x"].reshape(n, 3), "f": r["f"].reshape(n, 3), "type": r["type"].astype(np.int32),
         "mol": r["mol"], "tag": r["tag"], "box_lo": r["box"][:3], "box_hi": r["box"][3:],
         "periodic": np.ones(3, dtype=np.int32), "e_tersoff": r["e_tersoff"][0], "e_ilp": r["e_ilp"][0],
         "pvector": r["pvector"], "virial": r["virial"], "eatom": r["eatom"], "tap_flag": 0, "cut_global": 16.0,
         "skin": 2.0, "tersoff_file": "C.opt.tersoff", "tersoff_elements": "NULL C(O) C(O) C(O) C(O) C(O)",
         "ilp_elements": "C C C C C C"}
    if "min_counts" in r:
        d["min_counts"] = r["min_counts"]
        d["min_values"] = r["min_values"]
    if extra:
        d.update(extra)
    return d


def pack(s: S.System, r, tap_flag, extra=None):
    n = s.n
    d = {
        "x": r["x"].reshape(n, 3), "v": r["v"].reshape(n, 3), "f": r["f"].reshape(n, 3),
        "type": r["type"].astype(np.int32), "mol": r["mol"], "tag": r["tag"],
        "box_lo": r["box"][:3], "box_hi": r["box"][3:], "periodic": s.periodic.astype(np.int32),
        "e_tersoff": r["e_tersoff"][0], "e_ilp": r["e_ilp"][0], "pvector": r["pvector"],
        "virial": r["virial"], "eatom": r["eatom"], "tap_flag": tap_flag, "cut_global": 16.0,
        "skin": 2.0, "step": r["step"][0],
    }
    for k in ("vatom_tersoff", "vatom_ilp"):
        if k in r:
            d[k] = r[k].reshape(n, 6)
    if "tilt" in r:
        d["tilt"] = r["tilt"]
    if "nlist" in r:
        nl = r["nlist"].reshape(-1, 3)
        nl = nl[np.lexsort((nl[:, 2], nl[:, 1], nl[:, 0]))]
        d["nlist"] = nl.astype(np.int32)
        il = r["ilplist"].reshape(-1, 3)
        il = il[np.lexsort((il[:, 2], il[:, 1], il[:, 0]))]
        d["ilplist"] = il.astype(np.int32)
    if extra:
        d.update(extra)
    return d


ONLY = set(sys.argv[1:])     # optional: names of the fixtures to (re)generate


def want(*names) -> bool:
    return not ONLY or any(n in ONLY for n in names)


def save(name, d):
    if ONLY and name not in ONLY:
        return
    path = os.path.join(OUT, f"{name}.npz")
    np.savez_compressed(path, **d)
    print(f"{name}: {len(d['tag'])} atoms, {os.path.getsize(path) / 1024:.0f} KiB")


def main():
    if not os.path.exists(HARNESS):
        sys.exit("reference harness missing: make -f oracle/ref.mk REF=<reference> -j8")

    if want("bilayer_small", "bilayer_small_notaper"):
        _cases_bilayer_small()
    if want("hetero_small"):
        _case_hetero_small()
    if want("tiny_images", "edges", "trilayer_alt"):
        _cases_lists()
    if want("c1_t0", "c1_t100"):
        _cases_c1()
    if want("hetero_t20"):
        _case_hetero_t20()
    if want("case5016", "case5016_rep2", "case5016_min", "case5016_min_long"):
        _cases_case5016()
    if want("kc_bilayer", "kc_bilayer_notaper", "kc_trilayer_t30"):
        _cases_kc()
    if want("tri_bilayer", "tri_tilted_bn", "tri_small"):
        _cases_triclinic()


def _cases_bilayer_small():
    # 1. small AB bilayer graphene, displaced, thermal velocities; lists
    s = S.thermalize(S.displace(S.ab_bilayer_graphene(8, 5), 0.05, seed=11), 300.0, seed=12)
    save("bilayer_small", pack(s, run_reference(s, lists=True), 1))
    # 2. same structure with the taper off
    save("bilayer_small_notaper", pack(s, run_reference(s, tap_flag=0), 0))


def _case_hetero_small():
    # 3. twisted graphene/hBN bilayer (B, N, C parameters); lists
    s = S.displace(S.twisted_bilayer(8, 5, 3.0, top="hbn", spacing=3.3, shift=(0.4, 0.7)), 0.03, seed=21)
    save("hetero_small", pack(s, run_reference(s, lists=True), 1, {"strain_max": s.meta["strain_max"]}))


def _cases_lists():
    # 4. box shorter than the 18 A neighbour cutoff: several images of each atom; lists
    s = S.displace(S.ab_bilayer_graphene(6, 4), 0.04, seed=31)
    save("tiny_images", pack(s, run_reference(s, lists=True), 1))
    # 5. ribbon with free edges + isolated atoms: 0/1/2/3 intralayer neighbours; lists
    s = S.displace(S.flake_edges(4, 3), 0.03, seed=41)
    save("edges", pack(s, run_reference(s, lists=True), 1))
    # 6. three-layer graphite, alternating molecule ids (layers 1 and 3 share an id); lists
    s = S.displace(S.graphite_slab(3, 8, 5, spacing=3.35, mol_mode="alternate"), 0.04, seed=51)
    save("trilayer_alt", pack(s, run_reference(s, lists=True), 1))


def _cases_c1():
    # 7. the 7,200-atom plain-FP64 workload at t=0 and after 100 NVE steps (dt = 1 fs)
    c1 = S.thermalize(S.ab_bilayer_graphene(30, 30), 300.0, seed=1)
    r0 = run_reference(c1)
    save("c1_t0", pack(c1, r0, 1))
    r100 = run_reference(c1, nsteps=100)
    save("c1_t100", pack(c1, r100, 1, {"x0": r0["x"].reshape(-1, 3), "v0": r0["v"].reshape(-1, 3)}))


def _case_hetero_t20():
    # 8. short NVE on the hetero cell (exercises B/N masses and parameters)
    h = S.thermalize(S.twisted_bilayer(8, 5, 3.0, top="hbn", spacing=3.3, shift=(0.4, 0.7)), 300.0, seed=61)
    r0 = run_reference(h)
    r20 = run_reference(h, nsteps=20)
    save("hetero_t20", pack(h, r20, 1, {"x0": r0["x"].reshape(-1, 3), "v0": r0["v"].reshape(-1, 3),
                                        "f0": r0["f"].reshape(-1, 3)}))


def _cases_case5016():
    # 9. the reference's own case (Cases/case_5016: 6 graphene layers, 5016 atoms, layer 1
    #    excluded from Tersoff by NULL, taper off): read_data, then forces
    save("case5016", pack_case(run_case()))
    # 10. the same after `replicate 2 1 1` (molecule ids offset per copy, as LAMMPS does)
    save("case5016_rep2", pack_case(run_case("replicate 2 1 1")))
    # 11. the case's minimisation (in.replicate.ilp_tersoff:123-125): layer 1 held by
    #     setforce, CG with the quadratic line search, etol = ftol = 1e-5
    r0 = run_case()
    rm = run_case("group l1 type 1", "fix sf l1 setforce 0.0 0.0 0.0\nminimize 1.0e-5 1.0e-5 1000 10000",
                  flags=("min",))
    save("case5016_min", pack_case(rm, {"x0": r0["x"].reshape(-1, 3)}))
    # 12. the same minimisation run to a tight energy tolerance: 135 CG iterations
    rm = run_case("group l1 type 1", "fix sf l1 setforce 0.0 0.0 0.0\nminimize 1.0e-10 1.0e-3 300 3000",
                  flags=("min",))
    save("case5016_min_long", pack_case(rm, {"x0": r0["x"].reshape(-1, 3)}))


def _cases_kc():
    # 13-15. Kolmogorov-Crespi full (CC.KC-full) as the interlayer style: a displaced,
    #        thermal AB bilayer with and without the taper (without it the energy carries
    #        the reference's offset), and 30 NVE steps of a larger bilayer
    s = S.thermalize(S.displace(S.ab_bilayer_graphene(8, 5), 0.05, seed=71), 300.0, seed=72)
    save("kc_bilayer", pack(s, run_reference(s, interlayer="kc"), 1, {"interlayer": "kc"}))
    save("kc_bilayer_notaper", pack(s, run_reference(s, tap_flag=0, interlayer="kc"), 0, {"interlayer": "kc"}))
    k = S.thermalize(S.displace(S.graphite_slab(3, 12, 7, spacing=3.35, mol_mode="unique"), 0.03, seed=73), 300.0,
                     seed=74)
    r0 = run_reference(k, interlayer="kc")
    r30 = run_reference(k, nsteps=30, interlayer="kc")
    save("kc_trilayer_t30", pack(k, r30, 1, {"interlayer": "kc", "x0": r0["x"].reshape(-1, 3),
                                             "v0": r0["v"].reshape(-1, 3), "f0": r0["f"].reshape(-1, 3),
                                             "e0": r0["e_ilp"][0]}))


def _cases_triclinic():
    # 16-18. triclinic (hexagonal) cells: an AB bilayer (xy tilt, z not periodic), four
    #        alternating-id layers with B/N in a cell periodic in z with all three tilts
    #        (the stacking continues through the tilted z edge), and a 24-atom bilayer
    #        cell much smaller than the 18 A neighbour cutoff (many images per edge)
    s = S.thermalize(S.displace(S.hex_layers(8, 6), 0.05, seed=81), 300.0, seed=82)
    save("tri_bilayer", pack(s, run_reference(s), 1))
    t = S.displace(S.hex_layers(7, 5, nlayers=4, spacing=3.35, species="BN", mol_mode="alternate", periodic_z=True,
                                xz=0.37, yz=0.21), 0.03, seed=83)
    save("tri_tilted_bn", pack(t, run_reference(t), 1))
    u = S.displace(S.hex_layers(3, 2), 0.03, seed=84)
    save("tri_small", pack(u, run_reference(u), 1))


if __name__ == "__main__":
    main()
