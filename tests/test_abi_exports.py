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


def test_plan_queries_and_tile_setters_refuse_null_plans(library):
    """The tuning and hand-off entry points check their pointers before touching a plan (no GPU)."""
    EINVAL = 1
    vp, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
    out_p, out_i, out_n = vp(), i32(), i64()
    assert library.epsp_scgd0_sigma_device(None, C.byref(out_p), C.byref(out_n)) == EINVAL
    for get in ("epsp_ladder_gemm_persistent", "epsp_ladder_gemm_pair"):
        assert getattr(library, get)(None, C.byref(out_i)) == EINVAL, get
    for put in ("epsp_ladder_set_gemm_persistent", "epsp_ladder_set_gemm_pair"):
        assert getattr(library, put)(None, i32(1)) == EINVAL, put
    assert library.epsp_ladder_set_gemm_config(None, i32(256), i32(1), i32(32)) == EINVAL


def test_context_utilities_refuse_null_contexts(library):
    """The host-registration, kept-g2 and test-hook entry points check the context first (no GPU)."""
    EINVAL = 1
    vp, i32, u32, u64 = C.c_void_p, C.c_int32, C.c_uint32, C.c_uint64
    buf = C.create_string_buffer(64)
    library.epsp_host_register.argtypes = [vp, vp, u64]
    library.epsp_host_unregister.argtypes = [vp, vp]
    assert library.epsp_host_register(None, C.cast(buf, vp), u64(64)) == EINVAL
    assert library.epsp_host_unregister(None, C.cast(buf, vp)) == EINVAL
    assert library.epsp_ctx_keep_g2(None, i32(1)) == EINVAL
    assert library.epsp_test_g2_host_gather(None, i32(1)) == EINVAL
    assert library.epsp_test_gemm_stall(None, i32(0), u32(64)) == EINVAL


def test_header_declares_the_tensor_core_paths():
    text = open(HEADER).read()
    for name, value in (("EPSP_PATH_GEMM_BF16", 2), ("EPSP_PATH_GEMM_TF32", 3)):
        assert re.search(rf"{name}\s*=\s*{value}\b", text), name
    from epspectral_gb300 import abi
    assert abi.PATHS["gemm_tf32"] == 3 and abi.PATHS["gemm_bf16"] == 2


def test_device_sigma_refuses_to_outlive_its_run():
    """A DeviceSigma names its plan's Σ of one run: after another run or a close it raises (no GPU:
    a stand-in plan object with the two attributes it reads)."""
    import types
    from epspectral_gb300.results import DeviceSigma
    plan = types.SimpleNamespace(handle=C.c_void_p(1234), run_gen=3)
    d = DeviceSigma(plan, 0xABC0, (4, 2, 1), 3)
    assert d.valid() and d.ptr()
    plan.run_gen = 4
    assert not d.valid()
    with pytest.raises(ValueError):
        d.ptr()
    plan.run_gen, plan.handle = 3, C.c_void_p()
    with pytest.raises(ValueError):
        d.ptr()


def test_julia_shim_and_integration_name_only_declared_entry_points():
    """The Julia ccall shim and the integration guide call nothing the header does not declare."""
    decl = set(declared())
    jl = open(os.path.join(PKG, "julia", "EPSpectralGB300.jl")).read()
    used = set(re.findall(r":(epsp_[a-z0-9_]+)", jl))
    assert used and not (used - decl), sorted(used - decl)
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    types = set(re.findall(r"\b(epsp_[a-z0-9_]+)\b", re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)))
    named = set(re.findall(r"\b(epsp_[a-z0-9_]+)\s*\(", text)) | set(re.findall(r"`(epsp_[a-z0-9_]+)`", text))
    assert not (named - decl - types), sorted(named - decl - types)
