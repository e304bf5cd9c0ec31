"""The C-ABI library loads and exports every entry point that include/epspectral_gb300.h declares
(no compute call: this runs without a GPU). The library is built first if it is missing."""
import ctypes as C
import os
import re

import pytest

from conftest import PKG, ROOT

HEADER = os.path.join(ROOT, "include", "epspectral_gb300.h")


def declared():
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    return sorted(set(re.findall(r"\b(epsp_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def library():
    import sys
    sys.path.insert(0, PKG)
    import build as B
    path = B.build()
    return C.CDLL(path)


def test_header_declares_the_loops_and_the_warm_start():
    names = declared()
    for n in ("epsp_scgd0_run", "epsp_ladder_run", "epsp_ladder_apply", "epsp_scgd0_imsigma",
              "epsp_scgd0_imsigma_noalloc", "epsp_warmstart_train", "epsp_warmstart_grad"):
        assert n in names


def test_library_exports_every_declared_symbol(library):
    missing = [n for n in declared() if not hasattr(library, n)]
    assert not missing, missing


def test_context_creation_without_gpu_fails_cleanly(library):
    """With no device epsp_create returns a status (not a crash); on a GPU machine it succeeds."""
    h = C.c_void_p()
    st = library.epsp_create(C.byref(h), 0)
    if st == 0:
        library.epsp_destroy(h)
    else:
        assert st in (6, 7) and not h.value  # ECUDA or EUNSUPPORTED
