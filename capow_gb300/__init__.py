"""capow_gb300: GB300 (sm_103a) implementation of CAPOW's periodic-box power-spectrum path.

The product is the C-ABI library ``libcapow_gpu.so`` (declared in ``include/capow.h``) and
the ``capow`` command-line driver. This module is a thin ctypes mirror of that C ABI for
Python callers and tests. Inputs may be NumPy arrays (host: copied to the GPU inside the
call) or any object exposing ``data_ptr()`` on a CUDA device (e.g. torch tensors: passed
through as device pointers, resident in HBM).

There is no CPU fallback: if the compiled library is missing, importing the bindings raises.
Build it with ``python -m capow_gb300.build`` (or ``__graft_entry__.build()``).

Reference mapping (paths in the CAPOW source tree):
  Params / read_params     src/read_params.c:30-428   read_parameterfile, check_inputs
  PowerSpectrum()          src/main.c:1123-1251       create_grids
  PowerSpectrum.paint      src/read_data.c:32-179, 514-745
  PowerSpectrum.power      src/main.c:106-148, 211-225, 266-271, 302-468
  normalise                src/main.c:1019-1056       output_power arithmetic
"""
from __future__ import annotations

import ctypes
import dataclasses
import os
from typing import List, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libcapow_gpu.so")
DRIVER_PATH = os.path.join(HERE, "bin", "capow")

# status codes (capow.h)
OK, EINVAL, ENOMEM, ECUDA, EBOUNDS, ETIMEOUT, ESTATE, ECUFFT, ENOTSUP = range(9)
FP64, FP32_MIXED, FP32_DETERMINISTIC = 0, 1, 2
SPEC_REFERENCE, SPEC_DD, SPEC_DP, SPEC_PP = 0, 1, 2, 4
F32, F64 = 0, 1
FFT_AUTO, FFT_3D, FFT_ONE_LAUNCH = 0, 1, 2
PRECISIONS = {"fp64": FP64, "fp32": FP32_MIXED, "det": FP32_DETERMINISTIC}


class CapowError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(msg)
        self.status = status


class _Params(ctypes.Structure):
    _fields_ = [
        ("NX", ctypes.c_int), ("NY", ctypes.c_int), ("NZ", ctypes.c_int),
        ("XMIN", ctypes.c_double), ("XMAX", ctypes.c_double), ("YMIN", ctypes.c_double),
        ("YMAX", ctypes.c_double), ("ZMIN", ctypes.c_double), ("ZMAX", ctypes.c_double),
        ("InterpOrder", ctypes.c_int), ("DoInterlacing", ctypes.c_int),
        ("NK", ctypes.c_int), ("NMU", ctypes.c_int), ("Output2D", ctypes.c_int), ("OutputLog", ctypes.c_int),
        ("Mink", ctypes.c_double), ("Maxk", ctypes.c_double),
        ("Omega_m", ctypes.c_double), ("Redshift", ctypes.c_double),
        ("LOS", ctypes.c_int), ("Momentum", ctypes.c_int), ("Odd_Multipoles", ctypes.c_int),
    ]


class _Options(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("spectra", ctypes.c_int), ("device", ctypes.c_int),
                ("stream", ctypes.c_void_p), ("fft_path", ctypes.c_int), ("reserved", ctypes.c_int * 7)]


class _Particles(ctypes.Structure):
    _fields_ = [("n", ctypes.c_size_t), ("dtype", ctypes.c_int), ("on_device", ctypes.c_int),
                ("x", ctypes.c_void_p), ("y", ctypes.c_void_p), ("z", ctypes.c_void_p),
                ("vlos", ctypes.c_void_p), ("w", ctypes.c_void_p)]


class _Stats(ctypes.Structure):
    _fields_ = [("nread", ctypes.c_double), ("nout", ctypes.c_double), ("ngrid", ctypes.c_double),
                ("nsq", ctypes.c_double), ("vr", ctypes.c_double * 4), ("first_out_of_box", ctypes.c_int64)]


class _Grads(ctypes.Structure):
    _fields_ = [("on_device", ctypes.c_int), ("dtype", ctypes.c_int), ("dx", ctypes.c_void_p), ("dy", ctypes.c_void_p),
                ("dz", ctypes.c_void_p), ("dvlos", ctypes.c_void_p), ("dw", ctypes.c_void_p)]


class _Spectrum(ctypes.Structure):
    _fields_ = [("pk", ctypes.POINTER(ctypes.c_double) * 5), ("nmodes", ctypes.POINTER(ctypes.c_int64)),
                ("pk2d", ctypes.POINTER(ctypes.c_double)), ("nmodes2d", ctypes.POINTER(ctypes.c_int64)),
                ("shot", ctypes.c_double), ("norm", ctypes.c_double), ("alpha", ctypes.c_double),
                ("last_bin", ctypes.c_int), ("kind", ctypes.c_int)]


class _Mock(ctypes.Structure):
    _fields_ = [("params", _Params), ("parts", _Particles), ("out", ctypes.POINTER(_Spectrum)), ("status", ctypes.c_int)]


BATCH_GRAPH, BATCH_AUTOTUNE = 1, 2


class _SurveyParams(ctypes.Structure):
    _fields_ = [("Periodic", ctypes.c_int), ("Survey", ctypes.c_int), ("Coord_Type", ctypes.c_int),
                ("X_Origin", ctypes.c_double), ("Y_Origin", ctypes.c_double), ("Z_Origin", ctypes.c_double),
                ("REDMININ", ctypes.c_double), ("REDMAXIN", ctypes.c_double), ("NOBJ_Max", ctypes.c_longlong),
                ("NBAR_Column", ctypes.c_int), ("SkyArea", ctypes.c_double), ("FKP_Column", ctypes.c_int),
                ("FKP_Pk", ctypes.c_double), ("FKP_Pk_mom", ctypes.c_double), ("FKP_Pk_cross", ctypes.c_double)]


class _SurveyCatalogue(ctypes.Structure):
    _fields_ = [("n", ctypes.c_size_t), ("dtype", ctypes.c_int), ("on_device", ctypes.c_int),
                ("x", ctypes.c_void_p), ("y", ctypes.c_void_p), ("z", ctypes.c_void_p),
                ("w", ctypes.c_void_p), ("nbar", ctypes.c_void_p), ("pv", ctypes.c_void_p), ("pverr", ctypes.c_void_p)]


class _SurveyStats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in ("ngrid_data", "ngrid_rand", "data_nbw", "data_nbwsq", "data_nbsqwsq",
                                               "rand_nbw", "rand_nbwsq", "rand_nbsqwsq", "data_vr", "data_vrsq",
                                               "data_nbsqwsq_pv", "rand_nbsqwsq_pv")]


class _SurveyObjects(ctypes.Structure):
    _fields_ = [("n", ctypes.c_size_t), ("nread", ctypes.c_ulonglong)] + [
        (k, ctypes.POINTER(ctypes.c_float)) for k in ("x", "y", "z", "w", "nbar", "redshift", "pv", "pverr")] + [
        ("lo", ctypes.c_double * 3), ("hi", ctypes.c_double * 3), ("redmin", ctypes.c_double),
        ("redmax", ctypes.c_double), ("log", ctypes.c_void_p)]


# every entry point include/capow.h declares
EXPORTS = [
    "capow_create", "capow_paint", "capow_get_stats", "capow_power", "capow_normalise", "capow_num_spectra",
    "capow_copy_grid", "capow_stage_ms", "capow_kernel_launches", "capow_destroy", "capow_read_params",
    "capow_read_catalogue", "capow_free", "capow_write_output", "capow_bin_centre", "capow_strerror",
    "capow_last_error", "capow_paint_noalloc", "capow_backward", "capow_batch", "capow_tile_kernel_ms",
    "capow_batch_release", "capow_survey_create", "capow_survey_power", "capow_survey_copy_grid",
    "capow_survey_stage_ms", "capow_survey_kernel_launches", "capow_survey_last_error", "capow_survey_destroy",
    "capow_read_survey_params", "capow_read_survey", "capow_survey_objects_free", "capow_is_soa_catalogue",
    "capow_read_catalogue_soa", "capow_free_host", "capow_survey_nbar", "capow_abi_version",
    "capow_power_enqueue", "capow_power_result",
]

ABI_VERSION = 3  # the CAPOW_ABI_VERSION of include/capow.h that this mirror follows

_lib = None


def lib() -> ctypes.CDLL:
    """Load libcapow_gpu.so. Raises if it has not been built: there is no fallback."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing; build it with `python -m capow_gb300.build` "
                          "(the CUDA library is required: there is no CPU path)")
    L = ctypes.CDLL(LIB_PATH)
    L.capow_abi_version.restype = ctypes.c_int
    L.capow_abi_version.argtypes = []
    if L.capow_abi_version() != ABI_VERSION:
        raise ImportError(f"{LIB_PATH} has ABI version {L.capow_abi_version()}, this module follows {ABI_VERSION}: "
                          "rebuild it with `python -m capow_gb300.build`")
    vp, ip = ctypes.c_void_p, ctypes.c_int
    P, O = ctypes.POINTER(_Params), ctypes.POINTER(_Options)
    L.capow_create.argtypes = [P, O, ctypes.POINTER(vp)]
    L.capow_paint.argtypes = [vp, ctypes.POINTER(_Particles)]
    L.capow_paint_noalloc.argtypes = [vp, ctypes.POINTER(_Particles)]
    L.capow_get_stats.argtypes = [vp, ctypes.POINTER(_Stats)]
    L.capow_batch.argtypes = [ctypes.POINTER(_Mock), ip, O, ip]
    L.capow_batch_release.restype = None
    L.capow_batch_release.argtypes = []
    L.capow_backward.argtypes = [vp, ctypes.POINTER(ctypes.POINTER(ctypes.c_double)), ctypes.POINTER(_Grads)]
    L.capow_power.argtypes = [vp, ctypes.POINTER(_Spectrum), ip]
    L.capow_power_enqueue.argtypes = [vp]
    L.capow_power_result.argtypes = [vp, ctypes.POINTER(_Spectrum), ip]
    L.capow_normalise.argtypes = [P, ctypes.POINTER(_Spectrum)]
    L.capow_num_spectra.argtypes = [vp]
    L.capow_copy_grid.argtypes = [vp, ip, ctypes.POINTER(ctypes.c_double)]
    L.capow_stage_ms.argtypes = [vp, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                 ctypes.POINTER(ctypes.c_float)]
    L.capow_tile_kernel_ms.argtypes = [vp, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int64)]
    L.capow_kernel_launches.argtypes = [vp]
    L.capow_kernel_launches.restype = ctypes.c_int64
    L.capow_destroy.argtypes = [vp]
    L.capow_destroy.restype = None
    L.capow_read_params.argtypes = [ctypes.c_char_p, P, ctypes.c_char_p, ctypes.c_size_t]
    dpp = ctypes.POINTER(ctypes.POINTER(ctypes.c_double))
    L.capow_read_catalogue.argtypes = [ctypes.c_char_p, ip, ctypes.POINTER(ctypes.c_size_t), dpp, dpp, dpp, dpp,
                                       ctypes.c_char_p, ctypes.c_size_t]
    L.capow_free.argtypes = [vp]
    L.capow_free.restype = None
    L.capow_write_output.argtypes = [ctypes.c_char_p, P, ctypes.POINTER(_Spectrum)]
    L.capow_bin_centre.argtypes = [P, ip]
    L.capow_bin_centre.restype = ctypes.c_double
    L.capow_strerror.argtypes = [ip]
    L.capow_strerror.restype = ctypes.c_char_p
    L.capow_last_error.argtypes = [vp]
    L.capow_last_error.restype = ctypes.c_char_p
    SP = ctypes.POINTER(_SurveyParams)
    L.capow_survey_create.argtypes = [P, SP, O, ctypes.POINTER(vp)]
    L.capow_survey_power.argtypes = [vp, ctypes.POINTER(_SurveyCatalogue), ctypes.POINTER(_SurveyCatalogue),
                                     ctypes.POINTER(_Spectrum), ctypes.POINTER(_SurveyStats)]
    L.capow_survey_copy_grid.argtypes = [vp, ip, ctypes.POINTER(ctypes.c_double)]
    L.capow_survey_stage_ms.argtypes = [vp, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                        ctypes.POINTER(ctypes.c_int)]
    L.capow_survey_kernel_launches.argtypes = [vp]
    L.capow_survey_kernel_launches.restype = ctypes.c_int64
    L.capow_survey_last_error.argtypes = [vp]
    L.capow_survey_last_error.restype = ctypes.c_char_p
    L.capow_survey_destroy.argtypes = [vp]
    L.capow_survey_destroy.restype = None
    L.capow_read_survey_params.argtypes = [ctypes.c_char_p, P, SP, ctypes.c_char_p, ctypes.c_size_t]
    L.capow_read_survey.argtypes = [ctypes.c_char_p, P, SP, ip, ctypes.POINTER(_SurveyObjects), ctypes.c_char_p,
                                    ctypes.c_size_t]
    L.capow_survey_objects_free.argtypes = [ctypes.POINTER(_SurveyObjects)]
    L.capow_survey_objects_free.restype = None
    L.capow_is_soa_catalogue.argtypes = [ctypes.c_char_p]
    L.capow_read_catalogue_soa.argtypes = [ctypes.c_char_p, ip, ctypes.POINTER(ctypes.c_size_t),
                                           ctypes.POINTER(ip)] + [ctypes.POINTER(vp)] * 4 + [ctypes.c_char_p,
                                                                                             ctypes.c_size_t]
    L.capow_free_host.argtypes = [vp]
    L.capow_free_host.restype = None
    L.capow_survey_nbar.argtypes = [P, SP, ctypes.POINTER(_SurveyObjects), ctypes.POINTER(_SurveyObjects),
                                    ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p, ctypes.c_size_t]
    _lib = L
    return L


@dataclasses.dataclass
class Params:
    """capow_params: the run_parameters.dat tags of the periodic path (src/read_params.c:65-227)."""
    NX: int = 32
    NY: int = 32
    NZ: int = 32
    XMIN: float = 0.0
    XMAX: float = 1000.0
    YMIN: float = 0.0
    YMAX: float = 1000.0
    ZMIN: float = 0.0
    ZMAX: float = 1000.0
    InterpOrder: int = 2
    DoInterlacing: int = 1
    NK: int = 20
    NMU: int = 4
    Output2D: int = 0
    OutputLog: int = 0
    Mink: float = 0.0
    Maxk: float = 0.2
    Omega_m: float = 0.3089
    Redshift: float = 0.1
    LOS: int = 0
    Momentum: int = 0
    Odd_Multipoles: int = 0

    def to_c(self) -> _Params:
        return _Params(**{f.name: getattr(self, f.name) for f in dataclasses.fields(self)})

    @classmethod
    def from_c(cls, c: _Params) -> "Params":
        return cls(**{f.name: getattr(c, f.name) for f in dataclasses.fields(cls)})


def read_params(path: str) -> Params:
    """capow_read_params: the reference's parameter-file reader and checks."""
    c = _Params()
    msg = ctypes.create_string_buffer(8192)
    rc = lib().capow_read_params(path.encode(), ctypes.byref(c), msg, len(msg))
    if rc != OK:
        raise CapowError(rc, msg.value.decode())
    return Params.from_c(c)


def read_catalogue(path: str, los: int):
    """capow_read_catalogue: returns (x, y, z, vlos) float64 arrays."""
    L = lib()
    n = ctypes.c_size_t()
    ptrs = [ctypes.POINTER(ctypes.c_double)() for _ in range(4)]
    msg = ctypes.create_string_buffer(4096)
    rc = L.capow_read_catalogue(path.encode(), los, ctypes.byref(n), *[ctypes.byref(p) for p in ptrs], msg, len(msg))
    if rc != OK:
        raise CapowError(rc, msg.value.decode())
    out = []
    for p in ptrs:
        a = np.ctypeslib.as_array(p, shape=(n.value,)).copy() if n.value else np.zeros(0)
        L.capow_free(ctypes.cast(p, ctypes.c_void_p))
        out.append(a)
    return tuple(out)


SOA_MAGIC = b"CAPOWSOA"


def write_soa_catalogue(path: str, x, y, z, vx, vy, vz, dtype=np.float32) -> None:
    """Write a binary catalogue (include/capow.h: "CAPOWSOA", version 1, dtype, n, 6 columns, then the
    columns x, y, z, vx, vy, vz), which the `capow` driver reads in place of a text catalogue."""
    dt = np.dtype(dtype)
    if dt not in (np.float32, np.float64):
        raise ValueError("dtype must be float32 or float64")
    cols = [np.ascontiguousarray(c, dtype=dt) for c in (x, y, z, vx, vy, vz)]
    n = len(cols[0])
    if any(len(c) != n for c in cols):
        raise ValueError("columns differ in length")
    header = SOA_MAGIC + np.array([1, 1 if dt == np.float64 else 0], "<u4").tobytes() + \
        np.array([n], "<u8").tobytes() + np.array([6, 0], "<u4").tobytes()
    with open(path, "wb") as f:
        f.write(header)
        for c in cols:
            f.write(c.astype(dt.newbyteorder("<"), copy=False).tobytes())


def read_catalogue_soa(path: str, los: int):
    """capow_read_catalogue_soa: returns (x, y, z, vlos) arrays of the file's dtype."""
    L = lib()
    n, dt = ctypes.c_size_t(), ctypes.c_int()
    ptrs = [ctypes.c_void_p() for _ in range(4)]
    msg = ctypes.create_string_buffer(4096)
    rc = L.capow_read_catalogue_soa(path.encode(), los, ctypes.byref(n), ctypes.byref(dt),
                                    *[ctypes.byref(p) for p in ptrs], msg, len(msg))
    if rc != OK:
        raise CapowError(rc, msg.value.decode())
    ct = ctypes.c_double if dt.value == F64 else ctypes.c_float
    out = tuple(np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ct)), shape=(n.value,)).copy()
                if n.value else np.zeros(0, dtype=np.float64 if dt.value == F64 else np.float32) for p in ptrs)
    L.capow_free_host(ptrs[0])
    return out


def _ptr_of(a):
    """(address, dtype code, on_device, keepalive) for a numpy array or a CUDA tensor-like."""
    if a is None:
        return None, None, None, None
    if hasattr(a, "data_ptr") and hasattr(a, "is_cuda"):
        if not a.is_cuda:
            a = a.numpy()
        else:
            if not a.is_contiguous():
                raise ValueError("device arrays must be contiguous")
            name = str(a.dtype)
            code = F64 if "float64" in name else (F32 if "float32" in name else None)
            if code is None:
                raise ValueError("device arrays must be float32 or float64")
            return a.data_ptr(), code, 1, a
    arr = np.ascontiguousarray(a)
    if arr.dtype not in (np.float32, np.float64):
        arr = arr.astype(np.float64)
    return arr.ctypes.data, (F64 if arr.dtype == np.float64 else F32), 0, arr


class PowerSpectrum:
    """One capow context: paint a catalogue, then P_l(k) for the requested spectra.

    precision: "fp32" (FP32-mixed, default), "fp64" (plain double path), "det" (int64 fixed-point grids).
    fft_path:  "auto" (fused x-axis FFT + binning where it applies), "3d" (3-D cuFFT + binning kernel) or
               "one_launch" (as auto, with the z and y axes in one launch where NY and NZ are powers of two).
    spectra:   None -> one spectrum chosen by params.Momentum (one reference run); or any of
               ("dd", "dp", "pp") computed from one paint and one set of FFTs.
    """

    def __init__(self, params: Params, precision: str = "fp32", spectra=None, device: int = 0, stream=None,
                 fft_path: str = "auto"):
        self.params = params
        self._pc = params.to_c()
        mask = 0
        for s in (spectra or []):
            mask |= {"dd": SPEC_DD, "dp": SPEC_DP, "pp": SPEC_PP}[s]
        self.spectra_mask = mask
        opt = _Options(PRECISIONS[precision], mask, device, ctypes.c_void_p(stream or 0),
                       {"auto": FFT_AUTO, "3d": FFT_3D, "one_launch": FFT_ONE_LAUNCH}[fft_path])
        self._ctx = ctypes.c_void_p()
        rc = lib().capow_create(ctypes.byref(self._pc), ctypes.byref(opt), ctypes.byref(self._ctx))
        if rc != OK:
            err = self._err()
            self.close()
            raise CapowError(rc, f"capow_create: {lib().capow_strerror(rc).decode()}: {err}")
        self.nspec = lib().capow_num_spectra(self._ctx)
        self._keep = []
        self._keep_prev = []

    def _err(self) -> str:
        if not self._ctx:
            return ""
        return lib().capow_last_error(self._ctx).decode()

    def _check(self, rc: int, what: str):
        if rc != OK:
            raise CapowError(rc, f"{what}: {lib().capow_strerror(rc).decode()}: {self._err()}")

    def paint(self, x, y, z, vlos=None, w=None) -> None:
        parts = []
        for a in (x, y, z, vlos, w):
            parts.append(_ptr_of(a))
        codes = {p[1] for p in parts if p[0] is not None}
        devs = {p[2] for p in parts if p[0] is not None}
        if len(codes) != 1 or len(devs) != 1:
            raise ValueError("all particle arrays must share one dtype and one location")
        n = len(parts[0][3])
        for p in parts:
            if p[0] is not None and len(p[3]) != n:
                raise ValueError("particle arrays differ in length")
        # a host catalogue's copy may still be running when the next catalogue is painted behind a
        # pending power stage (power_enqueue): the previous paint's arrays stay referenced until then
        self._keep_prev = self._keep
        self._keep = [p[3] for p in parts]
        pc = _Particles(n, codes.pop(), devs.pop(), *[p[0] for p in parts])
        self._check(lib().capow_paint(self._ctx, ctypes.byref(pc)), "capow_paint")

    def paint_noalloc(self, x, y, z, vlos=None, w=None) -> None:
        """capow_paint_noalloc: the paint of an FP32 context from device-resident arrays, with no
        device allocation (its scratch is the library's fixed per-device array). For callers that
        cannot allocate at paint time; calls that overlap on the GPU share that array and race."""
        parts = [_ptr_of(a) for a in (x, y, z, vlos, w)]
        codes = {p[1] for p in parts if p[0] is not None}
        if len(codes) != 1 or any(p[2] != 1 for p in parts if p[0] is not None):
            raise ValueError("capow_paint_noalloc takes device arrays of one dtype")
        n = len(parts[0][3])
        if any(p[0] is not None and len(p[3]) != n for p in parts):
            raise ValueError("particle arrays differ in length")
        self._keep = [p[3] for p in parts]
        pc = _Particles(n, codes.pop(), 1, *[p[0] for p in parts])
        self._check(lib().capow_paint_noalloc(self._ctx, ctypes.byref(pc)), "capow_paint_noalloc")

    def stats(self) -> dict:
        s = _Stats()
        self._check(lib().capow_get_stats(self._ctx, ctypes.byref(s)), "capow_get_stats")
        return {"nread": s.nread, "nout": s.nout, "ngrid": s.ngrid, "nsq": s.nsq, "vr": list(s.vr),
                "first_out_of_box": s.first_out_of_box}

    def grid(self, which: int) -> np.ndarray:
        """Painted grid (0 A, 1 A interlaced, 2 B, 3 B interlaced) in the padded reference layout."""
        p = self.params
        n = p.NX * p.NY * 2 * (p.NZ // 2 + 1)
        out = np.zeros(n)
        self._check(lib().capow_copy_grid(self._ctx, which, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))),
                    "capow_copy_grid")
        return out

    def power(self) -> List[dict]:
        """Raw bin sums + shot/norm/alpha for each spectrum (capow_power)."""
        specs, bufs = self._spectrum_buffers()
        self._check(lib().capow_power(self._ctx, specs, self.nspec), "capow_power")
        return self._spectrum_dicts(specs, bufs)

    def power_enqueue(self) -> None:
        """capow_power_enqueue: queue the power stage of the painted catalogue and return at once. One
        paint() of the next catalogue may follow (its host copy overlaps this power stage) before
        power_result()."""
        self._check(lib().capow_power_enqueue(self._ctx), "capow_power_enqueue")

    def power_result(self) -> List[dict]:
        """capow_power_result: wait for the queued power stage; the same dicts as power()."""
        specs, bufs = self._spectrum_buffers()
        self._check(lib().capow_power_result(self._ctx, specs, self.nspec), "capow_power_result")
        return self._spectrum_dicts(specs, bufs)

    def _spectrum_buffers(self):
        p = self.params
        n2d = p.NK * p.NMU if p.Output2D else 0
        specs = (_Spectrum * self.nspec)()
        bufs = []
        for q in range(self.nspec):
            pk = [np.zeros(p.NK) for _ in range(5)]
            nm = np.zeros(p.NK, np.int64)
            p2 = np.zeros(max(n2d, 1))
            n2 = np.zeros(max(n2d, 1), np.int64)
            bufs.append((pk, nm, p2, n2))
            for l in range(5):
                specs[q].pk[l] = pk[l].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
            specs[q].nmodes = nm.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
            if n2d:
                specs[q].pk2d = p2.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
                specs[q].nmodes2d = n2.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
        return specs, bufs

    def _spectrum_dicts(self, specs, bufs) -> List[dict]:
        p = self.params
        n2d = p.NK * p.NMU if p.Output2D else 0
        out = []
        for q in range(self.nspec):
            pk, nm, p2, n2 = bufs[q]
            d = {"Pk0": pk[0], "Pk1": pk[1], "Pk2": pk[2], "Pk3": pk[3], "Pk4": pk[4], "Nmodes": nm,
                 "shot": specs[q].shot, "norm": specs[q].norm, "alpha": specs[q].alpha,
                 "kind": {0: "ref", SPEC_DD: "dd", SPEC_DP: "dp", SPEC_PP: "pp"}[specs[q].kind]}
            if n2d:
                d["Pk_2D"] = p2[:n2d]
                d["Nmodes_2D"] = n2[:n2d]
            out.append(d)
        return out

    def backward(self, dL_dP, out=None) -> dict:
        """capow_backward: gradients of a loss with respect to the last painted catalogue.

        dL_dP maps "Pk0".."Pk4" to arrays of NK (missing keys: zero) for a context with one spectrum,
        or is a list of such dicts, one per spectrum in the order power() returns them. Returns a dict
        of float64 host arrays dx, dy, dz, dvlos, dw; or pass `out`, a dict of contiguous device arrays
        (torch tensors) of the particles' dtype, to receive them on the device."""
        p = self.params
        per = [dL_dP] if isinstance(dL_dP, dict) else list(dL_dP)
        nspec = lib().capow_num_spectra(self._ctx)
        if len(per) != nspec:
            raise ValueError(f"backward needs dL/dP for each of the context's {nspec} spectra")
        arrs = [np.ascontiguousarray(d.get(f"Pk{l}", np.zeros(p.NK)), dtype=np.float64) for d in per for l in range(5)]
        ptrs = (ctypes.POINTER(ctypes.c_double) * len(arrs))(*[a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
                                                                for a in arrs])
        names = ("dx", "dy", "dz", "dvlos", "dw")
        if out is not None:
            t = next(iter(out.values()))
            code = F64 if "float64" in str(t.dtype) else F32
            g = _Grads(1, code, *[out[k].data_ptr() if k in out else None for k in names])
            self._check(lib().capow_backward(self._ctx, ptrs, ctypes.byref(g)), "capow_backward")
            return out
        keep = self._keep[0]
        n = len(keep)
        dt = np.float64 if ("float64" in str(keep.dtype)) else np.float32
        host = {k: np.zeros(n, dtype=dt) for k in names}
        g = _Grads(0, F64 if dt == np.float64 else F32, *[host[k].ctypes.data for k in names])
        self._check(lib().capow_backward(self._ctx, ptrs, ctypes.byref(g)), "capow_backward")
        return {k: v.astype(np.float64) for k, v in host.items()}

    def normalise(self, raw: dict) -> dict:
        """capow_normalise (output_power arithmetic) on a copy of one raw spectrum."""
        p = self.params
        d = {k: (np.array(v, copy=True) if isinstance(v, np.ndarray) else v) for k, v in raw.items()}
        s = _Spectrum()
        for l in range(5):
            s.pk[l] = d[f"Pk{l}"].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        s.nmodes = d["Nmodes"].ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
        if p.Output2D:
            s.pk2d = d["Pk_2D"].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
            s.nmodes2d = d["Nmodes_2D"].ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
        s.shot, s.norm = d["shot"], d["norm"]
        rc = lib().capow_normalise(ctypes.byref(self._pc), ctypes.byref(s))
        if rc != OK:
            raise CapowError(rc, "capow_normalise")
        d["last_bin"] = s.last_bin
        return d

    def stage_ms(self):
        a, b, c = ctypes.c_float(), ctypes.c_float(), ctypes.c_float()
        self._check(lib().capow_stage_ms(self._ctx, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)),
                    "capow_stage_ms")
        return a.value, b.value, c.value

    def tile_kernel_ms(self):
        """(device ms of the last FP32 paint's tile-deposit kernel, particle records it deposited)."""
        ms, rec = ctypes.c_float(), ctypes.c_int64()
        self._check(lib().capow_tile_kernel_ms(self._ctx, ctypes.byref(ms), ctypes.byref(rec)), "capow_tile_kernel_ms")
        return ms.value, rec.value

    def kernel_launches(self) -> int:
        return int(lib().capow_kernel_launches(self._ctx))

    def close(self):
        if getattr(self, "_ctx", None):
            lib().capow_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def run(params: Params, x, y, z, vlos=None, w=None, precision: str = "fp32", spectra=None, device: int = 0):
    """Paint + power in one call; returns the list of raw spectra dicts."""
    with PowerSpectrum(params, precision=precision, spectra=spectra, device=device) as ps:
        ps.paint(x, y, z, vlos, w)
        return ps.power()


def release_batch() -> None:
    """capow_batch_release: free the device state capow_batch keeps between calls."""
    lib().capow_batch_release()


def run_batch(mocks, precision: str = "fp32", spectra=None, graph: bool = False, autotune: bool = False,
              device: int = 0, stream=None):
    """capow_batch: many independent mocks in one call (the device state and graph of the batch are kept
    for a later call with the same mocks' parameters and sizes; release_batch frees them).

    mocks: list of (Params, (x, y, z, vlos, w)) with device arrays (vlos, w may be None).
    Returns a list of (status, [spectrum dict, ...]) in input order; the dicts hold raw sums as
    PowerSpectrum.power returns them (normalise with PowerSpectrum.normalise or capow_normalise)."""
    mask = 0
    for sp in (spectra or []):
        mask |= {"dd": SPEC_DD, "dp": SPEC_DP, "pp": SPEC_PP}[sp]
    nspec = 1 if mask == 0 else bin(mask).count("1")
    arr = (_Mock * len(mocks))()
    keep = []
    for i, (prm, parts) in enumerate(mocks):
        ptrs = [_ptr_of(a) for a in parts]
        codes = {q[1] for q in ptrs if q[0] is not None}
        if len(codes) != 1 or any(q[2] != 1 for q in ptrs if q[0] is not None):
            raise ValueError("capow_batch takes device arrays of one dtype per mock")
        n = len(ptrs[0][3])
        keep.append([q[3] for q in ptrs])
        specs = (_Spectrum * nspec)()
        bufs = []
        for q in range(nspec):
            pk = [np.zeros(prm.NK) for _ in range(5)]
            nm = np.zeros(prm.NK, np.int64)
            for l in range(5):
                specs[q].pk[l] = pk[l].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
            specs[q].nmodes = nm.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
            bufs.append((pk, nm))
        keep.append((specs, bufs))
        arr[i].params = prm.to_c()
        arr[i].parts = _Particles(n, codes.pop(), 1, *[q[0] for q in ptrs])
        arr[i].out = ctypes.cast(specs, ctypes.POINTER(_Spectrum))
    opt = _Options(PRECISIONS[precision], mask, device, ctypes.c_void_p(stream or 0), FFT_AUTO)
    flags = (BATCH_GRAPH if graph else 0) | (BATCH_AUTOTUNE if autotune else 0)
    rc = lib().capow_batch(arr, len(mocks), ctypes.byref(opt), flags)
    if rc != OK:
        raise CapowError(rc, f"capow_batch: {lib().capow_strerror(rc).decode()}")
    out = []
    for i in range(len(mocks)):
        specs, bufs = keep[2 * i + 1]
        res = []
        for q in range(nspec if arr[i].status == OK else 0):
            pk, nm = bufs[q]
            res.append({"Pk0": pk[0], "Pk1": pk[1], "Pk2": pk[2], "Pk3": pk[3], "Pk4": pk[4], "Nmodes": nm,
                        "shot": specs[q].shot, "norm": specs[q].norm, "alpha": specs[q].alpha,
                        "kind": {0: "ref", SPEC_DD: "dd", SPEC_DP: "dp", SPEC_PP: "pp"}[specs[q].kind]})
        out.append((arr[i].status, res))
    return out


# ---------------------------------------------------------------------------------------- survey mode
@dataclasses.dataclass
class SurveyParams:
    """capow_survey_params: the survey tags of run_parameters.dat (src/read_params.c:145-222)."""
    Periodic: int = 0
    Survey: int = 1
    Coord_Type: int = 0
    X_Origin: float = 0.0
    Y_Origin: float = 0.0
    Z_Origin: float = 0.0
    REDMININ: float = 0.0
    REDMAXIN: float = 10.0
    NOBJ_Max: int = 1 << 40
    NBAR_Column: int = 5
    SkyArea: float = 1.0
    FKP_Column: int = -1
    FKP_Pk: float = 5000.0
    FKP_Pk_mom: float = 0.0
    FKP_Pk_cross: float = 0.0

    def to_c(self) -> _SurveyParams:
        return _SurveyParams(**{f.name: getattr(self, f.name) for f in dataclasses.fields(self)})

    @classmethod
    def from_c(cls, c: _SurveyParams) -> "SurveyParams":
        return cls(**{f.name: getattr(c, f.name) for f in dataclasses.fields(cls)})


def read_survey_params(path: str):
    """capow_read_survey_params: (Params, SurveyParams) of a periodic or survey parameter file."""
    c, s = _Params(), _SurveyParams()
    msg = ctypes.create_string_buffer(8192)
    rc = lib().capow_read_survey_params(path.encode(), ctypes.byref(c), ctypes.byref(s), msg, len(msg))
    if rc != OK:
        raise CapowError(rc, msg.value.decode())
    return Params.from_c(c), SurveyParams.from_c(s)


def _read_survey_objects(path: str, params: Params, survey: SurveyParams, randoms: bool) -> _SurveyObjects:
    L = lib()
    o = _SurveyObjects()
    msg = ctypes.create_string_buffer(8192)
    pc, sc = params.to_c(), survey.to_c()
    rc = L.capow_read_survey(path.encode(), ctypes.byref(pc), ctypes.byref(sc), int(randoms), ctypes.byref(o), msg,
                             len(msg))
    if rc != OK:
        log = ctypes.string_at(o.log).decode() if o.log else ""
        L.capow_survey_objects_free(ctypes.byref(o))
        err = CapowError(rc, msg.value.decode())
        err.log = log
        raise err
    return o


def _survey_objects_dict(o: _SurveyObjects) -> dict:
    out = {k: (np.ctypeslib.as_array(getattr(o, k), shape=(o.n,)).copy() if o.n else np.zeros(0, np.float32))
           for k in ("x", "y", "z", "w", "nbar", "redshift", "pv", "pverr")}
    out.update(n=o.n, nread=o.nread, lo=list(o.lo), hi=list(o.hi), redmin=o.redmin, redmax=o.redmax,
               log=ctypes.string_at(o.log).decode() if o.log else "")
    return out


def read_survey(path: str, params: Params, survey: SurveyParams, randoms: bool) -> dict:
    """capow_read_survey: the objects read_survey_serial_ascii keeps (float32 arrays) and its counters."""
    o = _read_survey_objects(path, params, survey, randoms)
    out = _survey_objects_dict(o)
    lib().capow_survey_objects_free(ctypes.byref(o))
    return out


def read_survey_pair(data_path: str, rand_path: str, params: Params, survey: SurveyParams):
    """Both catalogues of a survey run as the reference's main reads them: capow_read_survey twice and,
    for NBAR_Column < 0, capow_survey_nbar (compute_nbar). Returns (data, randoms, printed nbar lines)."""
    L = lib()
    d = _read_survey_objects(data_path, params, survey, False)
    try:
        r = _read_survey_objects(rand_path, params, survey, True)
    except CapowError:
        L.capow_survey_objects_free(ctypes.byref(d))
        raise
    nlog = ""
    try:
        if survey.NBAR_Column < 0:
            pc, sc = params.to_c(), survey.to_c()
            logp = ctypes.c_void_p()
            msg = ctypes.create_string_buffer(4096)
            rc = L.capow_survey_nbar(ctypes.byref(pc), ctypes.byref(sc), ctypes.byref(d), ctypes.byref(r),
                                     ctypes.byref(logp), msg, len(msg))
            if logp.value:
                nlog = ctypes.string_at(logp.value).decode()
                L.capow_free(logp)
            if rc != OK:
                raise CapowError(rc, msg.value.decode())
        return _survey_objects_dict(d), _survey_objects_dict(r), nlog
    finally:
        L.capow_survey_objects_free(ctypes.byref(d))
        L.capow_survey_objects_free(ctypes.byref(r))


def _survey_cat(cat, velocities: bool):
    """A capow_survey_catalogue for a dict (or tuple) of x, y, z, w, nbar arrays and, with velocities, pv and
    pverr (numpy: host; CUDA tensors: device), plus the arrays to keep alive. A randoms catalogue may leave
    pv out (it is not read)."""
    keys = ("x", "y", "z", "w", "nbar") + (("pv", "pverr") if velocities else ())
    if isinstance(cat, dict):
        arrs = [cat.get(k) if k == "pv" else cat[k] for k in keys]
    else:
        arrs = list(cat)[:len(keys)]
        if len(arrs) != len(keys):
            raise ValueError(f"survey catalogue needs {', '.join(keys)}")
    given = [k for k, a in zip(keys, arrs) if a is not None]
    ptrs = [_ptr_of(a) for a in arrs if a is not None]
    codes = {p[1] for p in ptrs}
    devs = {p[2] for p in ptrs}
    if len(codes) != 1 or len(devs) != 1:
        raise ValueError("survey catalogue arrays must share one dtype and one location")
    n = len(ptrs[0][3])
    if any(len(p[3]) != n for p in ptrs):
        raise ValueError("survey catalogue arrays differ in length")
    where = dict(zip(given, (p[0] for p in ptrs)))
    addr = [where.get(k) for k in ("x", "y", "z", "w", "nbar", "pv", "pverr")]
    return _SurveyCatalogue(n, codes.pop(), devs.pop(), *addr), [p[3] for p in ptrs]


class SurveySpectrum:
    """One capow survey context (capow_survey_create): the survey estimator's P_l(k) from data and randoms.

    precision: "fp64" (plain double path) or "fp32" (FP32 grids and FFTs, FP64 sums and bins)."""

    def __init__(self, params: Params, survey: SurveyParams, precision: str = "fp64", device: int = 0, stream=None):
        self.params, self.survey = params, survey
        self._pc, self._sc = params.to_c(), survey.to_c()
        opt = _Options(PRECISIONS[precision], 0, device, ctypes.c_void_p(stream or 0), FFT_AUTO)
        self._ctx = ctypes.c_void_p()
        rc = lib().capow_survey_create(ctypes.byref(self._pc), ctypes.byref(self._sc), ctypes.byref(opt),
                                       ctypes.byref(self._ctx))
        if rc != OK:
            err = self._err()
            self.close()
            raise CapowError(rc, f"capow_survey_create: {lib().capow_strerror(rc).decode()}: {err}")

    def _err(self) -> str:
        return lib().capow_survey_last_error(self._ctx).decode() if self._ctx else ""

    def _check(self, rc: int, what: str):
        if rc != OK:
            raise CapowError(rc, f"{what}: {lib().capow_strerror(rc).decode()}: {self._err()}")

    def power(self, data, rand) -> dict:
        """Raw bin sums, Nmodes, shot, norm, alpha and the survey counters (capow_survey_power)."""
        p = self.params
        dc, keep_d = _survey_cat(data, p.Momentum != 0)
        rc_, keep_r = _survey_cat(rand, p.Momentum != 0)
        pk = [np.zeros(p.NK) for _ in range(5)]
        nm = np.zeros(p.NK, np.int64)
        n2d = p.NK * p.NMU if p.Output2D else 0
        p2, n2 = np.zeros(max(n2d, 1)), np.zeros(max(n2d, 1), np.int64)
        s = _Spectrum()
        for l in range(5):
            s.pk[l] = pk[l].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        s.nmodes = nm.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
        if n2d:
            s.pk2d = p2.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
            s.nmodes2d = n2.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
        st = _SurveyStats()
        self._check(lib().capow_survey_power(self._ctx, ctypes.byref(dc), ctypes.byref(rc_), ctypes.byref(s),
                                             ctypes.byref(st)), "capow_survey_power")
        del keep_d, keep_r
        out = {"Pk0": pk[0], "Pk1": pk[1], "Pk2": pk[2], "Pk3": pk[3], "Pk4": pk[4], "Nmodes": nm,
               "shot": s.shot, "norm": s.norm, "alpha": s.alpha, "kind": "ref",
               "stats": {k: getattr(st, k) for k, _ in _SurveyStats._fields_}}
        if n2d:
            out["Pk_2D"], out["Nmodes_2D"] = p2[:n2d], n2[:n2d]
        return out

    def normalise(self, raw: dict) -> dict:
        """capow_normalise (output_power arithmetic) on a copy of one raw spectrum."""
        p = self.params
        d = {k: (np.array(v, copy=True) if isinstance(v, np.ndarray) else v) for k, v in raw.items()}
        s = _Spectrum()
        for l in range(5):
            s.pk[l] = d[f"Pk{l}"].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        s.nmodes = d["Nmodes"].ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
        if p.Output2D:
            s.pk2d = d["Pk_2D"].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
            s.nmodes2d = d["Nmodes_2D"].ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
        s.shot, s.norm = d["shot"], d["norm"]
        rc = lib().capow_normalise(ctypes.byref(self._pc), ctypes.byref(s))
        if rc != OK:
            raise CapowError(rc, "capow_normalise")
        d["last_bin"] = s.last_bin
        return d

    def grid(self, which: int) -> np.ndarray:
        """A painted grid of the last evaluation, padded reference layout. which = stencil * fields + field:
        the density (field 0) and, for Momentum 2 and 3, the momentum grid (field 1); stencil 1 is the
        interlaced copy."""
        p = self.params
        out = np.zeros(p.NX * p.NY * 2 * (p.NZ // 2 + 1))
        self._check(lib().capow_survey_copy_grid(self._ctx, which,
                                                 out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))),
                    "capow_survey_copy_grid")
        return out

    def stage_ms(self):
        """(paint ms, multipole ms, FFT sets) of the last evaluation."""
        a, b, n = ctypes.c_float(), ctypes.c_float(), ctypes.c_int()
        self._check(lib().capow_survey_stage_ms(self._ctx, ctypes.byref(a), ctypes.byref(b), ctypes.byref(n)),
                    "capow_survey_stage_ms")
        return a.value, b.value, n.value

    def kernel_launches(self) -> int:
        return int(lib().capow_survey_kernel_launches(self._ctx))

    def close(self):
        if getattr(self, "_ctx", None):
            lib().capow_survey_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
