"""Host-side checks of the C ABI that need no GPU: the library loads and exports every
function include/lmff_gb300.h declares, and the potential-file parser reproduces the
reference's error behaviour (pair_tersoff.cpp:458-558, pair_ilp_graphene_hbn.cpp:311-381)."""
import ctypes as C
import os
import re

import pytest
from conftest import ILP, ROOT, TERSOFF

from lmff_gb300 import build, capi

HEADER = os.path.join(ROOT, "include", "lmff_gb300.h")


@pytest.fixture(scope="module")
def lib():
    build.build()
    return capi.load_library()


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(lmff_[a-z_]+)\s*\(", src)))


def test_header_declares_the_abi():
    names = declared_functions()
    for must in ("lmff_create", "lmff_compute", "lmff_compute_device", "lmff_upload", "lmff_run_nve",
                 "lmff_batch_set", "lmff_batch_compute", "lmff_export_list", "lmff_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_strerror_messages_match_reference(lib):
    assert b"too many neighbors" in lib.lmff_strerror(-4)
    assert b"normal vector is zero" in lib.lmff_strerror(-5)


def _create(lib, tersoff, ilp, elements=("C", "B", "N")):
    h = C.c_void_p()
    arr = (C.c_char_p * len(elements))(*[e.encode() for e in elements])
    rc = lib.lmff_create_from_files(C.byref(h), tersoff.encode() if tersoff else None,
                                    ilp.encode() if ilp else None, len(elements), arr, 16.0, 1, 2.0, 0)
    msg = lib.lmff_last_error(None).decode()
    if rc == 0:
        lib.lmff_destroy(h)
    return rc, msg


def test_good_files_parse(lib):
    rc, msg = _create(lib, TERSOFF, ILP)
    if lib.lmff_device_count() == 0:
        assert rc == -10 and "device" in msg      # parsed, then no GPU here
    else:
        assert rc == 0


def test_missing_file(lib, tmp_path):
    rc, msg = _create(lib, str(tmp_path / "nope.tersoff"), ILP)
    assert rc == -6 and "Cannot open Tersoff potential file" in msg


def test_tersoff_short_entry_is_format_error(lib, tmp_path):
    bad = tmp_path / "bad.tersoff"
    lines = open(TERSOFF).read().splitlines()
    out, done = [], False
    for ln in lines:
        if not done and ln.strip() and not ln.lstrip().startswith("#"):
            out.append(" ".join(ln.split()[:16]))   # drop one word of the first entry
            done = True
        else:
            out.append(ln)
    bad.write_text("\n".join(out) + "\n")
    rc, msg = _create(lib, str(bad), ILP)
    assert rc == -6 and "Incorrect format in Tersoff potential file" in msg


def test_tersoff_missing_entry(lib, tmp_path):
    bad = tmp_path / "miss.tersoff"
    keep = [ln for ln in open(TERSOFF).read().splitlines() if not ln.split()[:3] == ["C", "C", "C"]]
    bad.write_text("\n".join(keep) + "\n")
    rc, msg = _create(lib, str(bad), ILP)
    assert rc == -6 and "missing an entry" in msg


def test_tersoff_duplicate_entry(lib, tmp_path):
    bad = tmp_path / "dup.tersoff"
    lines = open(TERSOFF).read().splitlines()
    cc = [ln for ln in lines if ln.split()[:3] == ["C", "C", "C"]]
    bad.write_text("\n".join(lines + cc) + "\n")
    rc, msg = _create(lib, str(bad), ILP)
    assert rc == -6 and "duplicate entry" in msg


def test_tersoff_illegal_parameter(lib, tmp_path):
    bad = tmp_path / "ill.tersoff"
    out = []
    for ln in open(TERSOFF).read().splitlines():
        w = ln.split()
        if w[:3] == ["C", "C", "C"]:
            w[3] = "2.0"          # m must be 1 or 3 (pair_tersoff.cpp:522-524)
            ln = " ".join(w)
        out.append(ln)
    bad.write_text("\n".join(out) + "\n")
    rc, msg = _create(lib, str(bad), ILP)
    assert rc == -6 and "Illegal Tersoff parameter" in msg


def test_ilp_missing_entry(lib, tmp_path):
    bad = tmp_path / "miss.ILP"
    keep = [ln for ln in open(ILP).read().splitlines() if ln.split()[:2] != ["B", "N"]]
    bad.write_text("\n".join(keep) + "\n")
    rc, msg = _create(lib, TERSOFF, str(bad))
    assert rc == -6 and "missing an entry" in msg


def test_ilp_short_entry(lib, tmp_path):
    bad = tmp_path / "short.ILP"
    out = []
    for ln in open(ILP).read().splitlines():
        w = ln.split()
        if w[:2] == ["C", "C"]:
            ln = " ".join(w[:12])
        out.append(ln)
    bad.write_text("\n".join(out) + "\n")
    rc, msg = _create(lib, TERSOFF, str(bad))
    assert rc == -6 and "ILP potential file" in msg


def test_null_elements_parse(lib):
    # types mapped to NULL are skipped by the element list (pair_tersoff.cpp:320-324)
    rc, msg = _create(lib, TERSOFF, ILP, elements=("C", "NULL", "C"))
    assert rc in (0, -10), msg
