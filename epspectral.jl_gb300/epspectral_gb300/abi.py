"""ctypes mirror of the C ABI in include/epspectral_gb300.h.

The structs below must match the header field for field. `ModelArrays.to_struct` turns the numpy
arrays of a setup (the reference's `setup` NamedTuple, src/scgd0.jl:173-183, plus the ladder's R
and v, src/ladder.jl:153-157) into an `epsp_model` whose pointers stay valid while the
`ModelArrays` object lives.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

EPSP_OK = 0
EPSP_EINVAL = 1
EPSP_ENOMEM = 2
EPSP_ENOROOT_MU = 3
EPSP_ENOTCONV = 4
EPSP_EDEVICE_TIMEOUT = 5
EPSP_ECUDA = 6
EPSP_EUNSUPPORTED = 7

STATUS_NAMES = {
    EPSP_OK: "OK", EPSP_EINVAL: "EINVAL", EPSP_ENOMEM: "ENOMEM", EPSP_ENOROOT_MU: "ENOROOT_MU",
    EPSP_ENOTCONV: "ENOTCONV", EPSP_EDEVICE_TIMEOUT: "EDEVICE_TIMEOUT", EPSP_ECUDA: "ECUDA",
    EPSP_EUNSUPPORTED: "EUNSUPPORTED",
}

EPSP_F64, EPSP_F32, EPSP_BF16 = 0, 1, 2
EPSP_METAL, EPSP_SEMICONDUCTOR = 0, 1
EPSP_PATH_DIRECT_FP64, EPSP_PATH_GEMM_FP64, EPSP_PATH_GEMM_BF16, EPSP_PATH_GEMM_TF32 = 0, 1, 2, 3
EPSP_SOLVER_GMRES, EPSP_SOLVER_FIXED_POINT = 0, 1

PATHS = {"direct_fp64": EPSP_PATH_DIRECT_FP64, "gemm_fp64": EPSP_PATH_GEMM_FP64,
         "gemm_bf16": EPSP_PATH_GEMM_BF16, "gemm_tf32": EPSP_PATH_GEMM_TF32}

c_double_p = C.POINTER(C.c_double)
c_int32_p = C.POINTER(C.c_int32)
c_int64_p = C.POINTER(C.c_int64)
c_uint8_p = C.POINTER(C.c_uint8)


class epsp_grid(C.Structure):
    _fields_ = [("origin", C.c_double), ("unit", C.c_double), ("offsets", c_int64_p),
                ("n", C.c_int64)]


class epsp_model(C.Structure):
    _fields_ = [
        ("nm", C.c_int64), ("ni", C.c_int64), ("nf", C.c_int64),
        ("g2_dtype", C.c_int32), ("reserved0", C.c_int32), ("g2", C.c_void_p),
        ("nq", C.c_int64), ("omega_ph", c_double_p),
        ("nk_i", C.c_int64), ("nk_f", C.c_int64), ("iq_kk", c_int32_p),
        ("iks_i", c_int32_p), ("iks_f", c_int32_p),
        ("eps_i", c_double_p), ("w_i", c_double_p), ("eps_f", c_double_p), ("w_f", c_double_p),
        ("f_to_i", c_int32_p),
        ("nmult", C.c_int64), ("mult_ptr", c_int32_p), ("mult_idx", c_int32_p),
        ("omegas", epsp_grid), ("omegas_spectral", epsp_grid),
        ("W", C.c_double), ("nstates_base", C.c_double),
        ("R", c_double_p), ("v", c_double_p),
    ]


class epsp_options(C.Structure):
    _fields_ = [("path", C.c_int32), ("verbosity", C.c_int32), ("gpu_tile", C.c_int64),
                ("omega_acoustic", C.c_double)]


class epsp_occ(C.Structure):
    _fields_ = [("nT", C.c_int64), ("Tlist", c_double_p), ("nlist", c_double_p),
                ("nelec", C.c_double), ("spin_degeneracy", C.c_double), ("type", C.c_int32),
                ("reserved0", C.c_int32)]


class epsp_scgd0_history(C.Structure):
    _fields_ = [("err", c_double_p), ("mu", c_double_p), ("min_spectral_weight", c_double_p),
                ("wall", c_double_p), ("iter_frozen", c_int32_p), ("niter", C.c_int32),
                ("reserved0", C.c_int32)]


class epsp_ladder_history(C.Structure):
    _fields_ = [("norms", c_double_p), ("nnorms", c_int32_p), ("sigma_iter", c_double_p),
                ("nsigma", c_int32_p)]


def ptr(a: np.ndarray | None, ctype=C.c_double):
    """A ctypes pointer to the data of a contiguous numpy array (None -> NULL)."""
    if a is None:
        return C.POINTER(ctype)()
    assert a.flags["F_CONTIGUOUS"] or a.flags["C_CONTIGUOUS"], "array must be contiguous"
    return a.ctypes.data_as(C.POINTER(ctype))


def fortran(a, dtype) -> np.ndarray:
    """Column-major copy (or view) of `a` with `dtype`: the reference's Julia layout."""
    return np.asfortranarray(np.asarray(a, dtype=dtype))


class GridArrays:
    """Keeps the offsets of a FrequencyGrid alive behind an `epsp_grid`."""

    def __init__(self, grid):
        self.offsets = np.ascontiguousarray(grid.offsets, dtype=np.int64)
        self.struct = epsp_grid(float(grid.origin), float(grid.unit), ptr(self.offsets, C.c_int64),
                                len(self.offsets))


class ModelArrays:
    """The arrays of a setup in ABI layout, and the `epsp_model` that points at them."""

    def __init__(self, setup):
        s = setup
        g2 = s["g2"]
        if g2.dtype == np.float64:
            self.g2, self.g2_dtype = fortran(g2, np.float64), EPSP_F64
        elif g2.dtype == np.float32:
            self.g2, self.g2_dtype = fortran(g2, np.float32), EPSP_F32
        elif g2.dtype == np.uint16:  # bfloat16 bit patterns
            self.g2, self.g2_dtype = fortran(g2, np.uint16), EPSP_BF16
        else:
            raise TypeError(f"g2 must be float64, float32 or bfloat16 bits (uint16), got {g2.dtype}")
        nm, ni, nf = self.g2.shape
        self.omega_ph = fortran(s["omega_ph"], np.float64)
        self.iq_kk = fortran(s["iq_kk"], np.int32)
        self.iks_i = fortran(s["iks_i"], np.int32)
        self.iks_f = fortran(s["iks_f"], np.int32)
        self.eps_i = fortran(s["eps_i"], np.float64)
        self.w_i = fortran(s["w_i"], np.float64)
        self.eps_f = fortran(s["eps_f"], np.float64)
        self.w_f = fortran(s["w_f"], np.float64)
        self.f_to_i = fortran(s["f_to_i"], np.int32)
        mults = s.get("multiplets", [])
        self.mult_ptr = np.zeros(len(mults) + 1, dtype=np.int32)
        for k, m in enumerate(mults):
            self.mult_ptr[k + 1] = self.mult_ptr[k] + len(m)
        self.mult_idx = (np.concatenate([np.asarray(m, dtype=np.int32) for m in mults])
                         if mults else np.zeros(1, dtype=np.int32))
        self.grid = GridArrays(s["omegas"])
        self.grid_sp = GridArrays(s["omegas_spectral"])
        self.R = fortran(s["R"], np.float64) if s.get("R") is not None else None
        self.v = fortran(s["v"], np.float64) if s.get("v") is not None else None
        st = epsp_model()
        st.nm, st.ni, st.nf = nm, ni, nf
        st.g2_dtype = self.g2_dtype
        st.g2 = self.g2.ctypes.data_as(C.c_void_p)
        st.nq = self.omega_ph.shape[1]
        st.omega_ph = ptr(self.omega_ph)
        st.nk_i, st.nk_f = self.iq_kk.shape
        st.iq_kk = ptr(self.iq_kk, C.c_int32)
        st.iks_i = ptr(self.iks_i, C.c_int32)
        st.iks_f = ptr(self.iks_f, C.c_int32)
        st.eps_i, st.w_i = ptr(self.eps_i), ptr(self.w_i)
        st.eps_f, st.w_f = ptr(self.eps_f), ptr(self.w_f)
        st.f_to_i = ptr(self.f_to_i, C.c_int32)
        st.nmult = len(mults)
        st.mult_ptr = ptr(self.mult_ptr, C.c_int32)
        st.mult_idx = ptr(self.mult_idx, C.c_int32)
        st.omegas = self.grid.struct
        st.omegas_spectral = self.grid_sp.struct
        st.W = float(s["W"])
        st.nstates_base = float(s["nstates_base"])
        st.R = ptr(self.R)
        st.v = ptr(self.v)
        self.struct = st
        self.nm, self.ni, self.nf = nm, ni, nf
        self.nw = len(self.grid.offsets)
        self.nwa = len(self.grid_sp.offsets)


class OccArrays:
    """An `epsp_occ` for (Tlist, nlist, nelec, spin_degeneracy, type)."""

    def __init__(self, occ):
        self.Tlist = np.ascontiguousarray(occ["Tlist"], dtype=np.float64)
        self.nlist = np.ascontiguousarray(np.broadcast_to(occ.get("nlist", 0.0), self.Tlist.shape),
                                          dtype=np.float64)
        t = occ.get("type", "metal")
        typ = {"metal": EPSP_METAL, "semiconductor": EPSP_SEMICONDUCTOR}[t] if isinstance(t, str) else int(t)
        self.struct = epsp_occ(len(self.Tlist), ptr(self.Tlist), ptr(self.nlist),
                               float(occ.get("nelec", 0.0)), float(occ.get("spin_degeneracy", 2.0)),
                               typ, 0)
