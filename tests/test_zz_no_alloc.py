"""The allocation-free Fan-Migdal entry point against the plan-based one, on the GPU.

epsp_scgd0_imsigma_noalloc exists for callers that cannot allocate device memory (a Julia host
whose CUDA.jl pool or ElectronPhonon backend owns the device budget, code running where a
cudaMalloc is refused): they pass device pointers they already own and the library keeps its few
tables in a fixed static device array. Here the caller's buffers come from torch; the result of two
calls in a row must equal epsp_scgd0_imsigma of a DIRECT_FP64 plan on the same inputs to 1e-13
relative (the tolerance of the Fan-Migdal GPU test). This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

import refimpl as R
from epspectral_gb300 import FrequencyGrid
from epspectral_gb300.abi import GridArrays, epsp_grid

pytestmark = pytest.mark.gpu


def _bind(lib):
    fn = lib.epsp_scgd0_imsigma_noalloc
    i64, d, p = C.c_int64, C.c_double, C.c_void_p
    fn.restype = C.c_int
    fn.argtypes = [p, i64, i64, i64, p, i64, p, i64, i64, p, p, p, p, p, p, C.POINTER(epsp_grid), d, p, d, d, p]
    return fn


def test_noalloc_matches_plan_path():
    torch = pytest.importorskip("torch")
    from epspectral_gb300 import api
    from test_oracle_scgd0 import per_pair_setup
    lib = api.lib()
    fn = _bind(lib)
    nm, ni, nf = 3, 13, 17
    g = FrequencyGrid.from_nodes(np.concatenate([np.arange(-1.0, -0.5999, 0.02), np.arange(-0.5, 0.5001, 0.1),
                                                 np.arange(0.6, 1.0001, 0.02)]))
    nw = len(g)
    Sin = 0.1 * R.pseudorandom(nw, ni, seed=7) + 1j * (-0.05 - 0.05 * np.abs(R.pseudorandom(nw, ni, seed=8)))
    g2 = np.abs(R.pseudorandom(nm, ni, nf, seed=9))
    wq = 0.05 + 0.2 * np.abs(R.pseudorandom(nm, ni, nf, seed=10))
    wq[1, 2, :] = 0.0
    g2[1, 2, :] = np.inf
    s = per_pair_setup(g, g2, wq, 0.8 * R.pseudorandom(nf, seed=11),
                       np.array([(5 * (f + 1)) % ni for f in range(nf)], dtype=np.int32), np.full(nf, 1.0 / nf))
    mu, T, w_ac = 0.07, 0.03, 1e-3
    ctx = api.Context(0)
    ref = api.Scgd0Plan(s, path="direct_fp64", omega_acoustic=w_ac, ctx=ctx).imsigma(Sin, mu, T, np.full((nw, ni), 0.5))

    dev = torch.device("cuda:0")

    def on_dev(a, dtype):
        return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=dtype).ravel(order="F"))).to(dev)

    d_g2 = on_dev(s["g2"], np.float64)
    d_wph = on_dev(s["omega_ph"], np.float64)
    d_iq = on_dev(s["iq_kk"], np.int32)
    d_iksi, d_iksf = on_dev(s["iks_i"], np.int32), on_dev(s["iks_f"], np.int32)
    d_eps, d_wf, d_fti = on_dev(s["eps_f"], np.float64), on_dev(s["w_f"], np.float64), on_dev(s["f_to_i"], np.int32)
    d_sin = on_dev(np.ascontiguousarray(Sin.ravel(order="F")).view(np.float64), np.float64)  # interleaved re, im
    ga = GridArrays(g)
    nq = s["omega_ph"].shape[1]
    nk_i, nk_f = s["iq_kk"].shape
    torch.cuda.synchronize()
    for call in range(2):
        d_out = on_dev(np.full((nw, ni), 0.5), np.float64)
        torch.cuda.synchronize()
        st = fn(ctx.handle, nm, ni, nf, d_g2.data_ptr(), nq, d_wph.data_ptr(), nk_i, nk_f, d_iq.data_ptr(),
                d_iksi.data_ptr(), d_iksf.data_ptr(), d_eps.data_ptr(), d_wf.data_ptr(), d_fti.data_ptr(),
                C.byref(ga.struct), w_ac, d_sin.data_ptr(), mu, T, d_out.data_ptr())
        assert st == 0, lib.epsp_last_error(ctx.handle)
        got = d_out.cpu().numpy().reshape(nw, ni, order="F")
        assert np.all(np.isfinite(got))
        assert np.linalg.norm(got - ref) <= 1e-13 * np.linalg.norm(ref), call
    # a grid beyond the stated maximum is refused, with the reason
    big = GridArrays(FrequencyGrid(0.0, 1.0, np.arange(70000)))
    st = fn(ctx.handle, nm, ni, nf, d_g2.data_ptr(), nq, d_wph.data_ptr(), nk_i, nk_f, d_iq.data_ptr(),
            d_iksi.data_ptr(), d_iksf.data_ptr(), d_eps.data_ptr(), d_wf.data_ptr(), d_fti.data_ptr(),
            C.byref(big.struct), w_ac, d_sin.data_ptr(), mu, T, d_out.data_ptr())
    assert st == 1 and b"at most" in lib.epsp_last_error(ctx.handle)
    # offsets spread over ±2^62 with a gap of 1: the bucket count is clamped before its conversion to
    # an integer, so the table size is refused (no overflow) and nothing reaches the device
    wide = GridArrays(FrequencyGrid(0.0, 1.0, np.array([-(2 ** 62), -(2 ** 62) + 1, 2 ** 62], dtype=np.int64)))
    st = fn(ctx.handle, nm, ni, nf, d_g2.data_ptr(), nq, d_wph.data_ptr(), nk_i, nk_f, d_iq.data_ptr(),
            d_iksi.data_ptr(), d_iksf.data_ptr(), d_eps.data_ptr(), d_wf.data_ptr(), d_fti.data_ptr(),
            C.byref(wide.struct), w_ac, d_sin.data_ptr(), mu, T, d_out.data_ptr())
    assert st == 1 and b"at most" in lib.epsp_last_error(ctx.handle)
