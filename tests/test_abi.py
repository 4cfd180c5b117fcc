"""The C ABI library builds, loads and exports every entry point declared in
include/emst.h (no GPU needed: nothing here launches a kernel)."""
import ctypes
import os
import re
import shutil

import pytest

import emst_gb300


def _built():
    if not os.path.exists(emst_gb300.LIB_PATH):
        if shutil.which("nvcc") is None:
            pytest.skip("nvcc not available")
        emst_gb300.build()
    return ctypes.CDLL(emst_gb300.LIB_PATH)


def test_library_exports_every_declared_symbol():
    L = _built()
    syms = emst_gb300.declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing


def test_status_codes_match_header():
    txt = open(emst_gb300.HEADER).read()
    for code, name in emst_gb300.STATUS.items():
        assert ("%s = %d" % (name, code)) in txt


def test_header_constants_match_the_binding():
    import re
    txt = open(emst_gb300.HEADER).read()
    assert int(re.search(r"#define EMST_ROUND1_NEIGHBOURS (\d+)", txt).group(1)) == emst_gb300.ROUND1_NEIGHBOURS
    assert int(re.search(r"#define EMST_PROPOSAL_WEIGHTS (\d+)", txt).group(1)) == emst_gb300.PROPOSAL_WEIGHTS


def test_profile_struct_matches_header():
    # the ctypes mirror has one field per emst_profile member, in order
    txt = open(emst_gb300.HEADER).read()
    body = txt[txt.index("typedef struct {", txt.index("ms_grid") - 200):txt.index("} emst_profile;")]
    names = re.findall(r"^\s*(?:double|int64_t)\s+(\w+);", body, re.M)
    assert names == [f for f, _ in emst_gb300.Profile._fields_]


def test_null_context_is_rejected_without_touching_the_gpu():
    _built()
    L = emst_gb300.lib()
    assert L.emst_destroy(None) == 0
    assert L.emst_run(None) == 1  # EMST_EINVAL
    assert L.emst_last_error(None) == b"null context"
