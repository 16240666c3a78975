"""CPU checks of the C ABI library: it loads, exports everything include/*.h
declares, and refuses politely without a GPU (no compute calls here)."""
import ctypes

import pytest


def test_exports_every_declared_symbol(mf):
    lib = mf.load()
    declared = mf.declared_symbols()
    assert len(declared) >= 25
    missing = [n for n in declared if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version_and_strings(mf):
    lib = mf.load()
    assert lib.mf_abi_version() == 4
    assert lib.mf_status_string(0) == b"MF_OK"
    assert lib.mf_status_string(5) == b"MF_ERR_TIMEOUT"


def test_null_arguments_rejected(mf):
    lib = mf.load()
    assert lib.mf_create(None, None) == 1
    assert lib.mf_solve(None, 10, None, None) == 1
    assert lib.mf_destroy(None) == 0


def test_create_without_gpu(mf):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import numpy as np
    g = np.zeros((2, 3), np.float32)
    g[1, 0] = 1
    with pytest.raises(mf.MFError) as e:
        mf.Solver(2, 1.0, 1.0, 1.0, 1.0, [0, 1, 0], None, None, g)
    assert e.value.status == 7  # MF_ERR_UNSUPPORTED


def _header():
    import os
    import re
    here = os.path.dirname(os.path.abspath(__file__))
    text = open(os.path.join(os.path.dirname(here), "include", "mf.h")).read()
    return re.sub(r"/\*.*?\*/", "", text, flags=re.S)


def _enum(name):
    import re
    body = re.search(r"typedef enum %s \{(.*?)\} %s;" % (name, name), _header(), re.S).group(1)
    return {k: int(v) for k, v in re.findall(r"(MF_\w+)\s*=\s*(-?\d+)", body)}


def _struct_fields(name):
    import re
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), _header(), re.S).group(1)
    out = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        ctype, names = decl.split(None, 1) if not decl.startswith("const ") else decl[6:].split(None, 1)
        for nm in names.split(","):
            nm = nm.strip().lstrip("*")
            arr = re.match(r"(\w+)\[(\d+)\]", nm)
            out.append((arr.group(1), int(arr.group(2))) if arr else (nm, 1))
    return out


def test_python_tables_match_the_header(mf):
    # The binding's option, quantity, kernel-kind and status tables carry the
    # header's enum values: a new enumerator needs its binding entry.
    opt = _enum("mf_option")
    assert {("MF_OPT_" + k.upper()): v for k, v in mf.OPT.items()} == opt
    # quantities are named after the reference's members (magnetic_bodyforce
    # is MF_Q_FORCE): the values must be the header's, one to one
    q = _enum("mf_quantity")
    assert sorted(mf.Q.values()) == sorted(q.values())
    kk = _enum("mf_kernel_kind")
    assert {("MF_K_" + k.upper()): v for k, v in mf.KERNEL.items()} == kk
    st = _enum("mf_status")
    assert {v: k for k, v in st.items()} == mf.STATUS


@pytest.mark.parametrize("name", ["mf_counters", "mf_kernel_stats", "mf_fmm_stats", "mf_scene_desc",
                                  "mf_server_config", "mf_server_stats"])
def test_ctypes_structs_match_the_header(mf, name):
    # Field names and order of every ctypes mirror agree with the header.
    ours = [(f[0], getattr(f[1], "_length_", 1)) for f in getattr(mf, name)._fields_]
    assert ours == _struct_fields(name)
