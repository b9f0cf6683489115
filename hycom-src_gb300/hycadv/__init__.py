"""hycadv -- Python mirror of HYCOM's tracer-advection interface over libhycadv.

The reference routines and the functions here that stand in for them
(same names, argument meaning and order):

=====================================  ==========================================
reference (HYCOM-src)                  here
=====================================  ==========================================
``tsadvc(m,n)``  mod_tsadvc.F90:1708   :meth:`Context.tsadvc`
``advem(...)``   mod_tsadvc.F90:69     :meth:`Context.advem`
``xctilr(...)``  mod_xc_sm.h:1337      :meth:`Context.xctilr`
``bigrid(...)``  bigrid.F90:1          :func:`bigrid`
=====================================  ==========================================

Everything calls the CUDA library through its C ABI (include/hycom_adv.h)
with ctypes; there is no CPU implementation behind these functions, and a
missing or unloadable library raises :class:`HycError`.

Array layout is the reference's: a 2-D slice is a C-contiguous array of
shape (jdm+2*nbdy, idm+2*nbdy) (Fortran column-major (ld1, ld2)).  Arrays on
the host are numpy float64; arrays on the GPU are torch float64 CUDA tensors.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libhycadv.so")

HYC_OK = 0
ERRORS = {-1: "HYC_ERR_ARG", -2: "HYC_ERR_ADVTYP", -3: "HYC_ERR_NBDY", -4: "HYC_ERR_MASK", -5: "HYC_ERR_CUDA",
          -6: "HYC_ERR_FIELD", -7: "HYC_ERR_GRID", -8: "HYC_ERR_UNSUPPORTED", -9: "HYC_ERR_NOMEM",
          -10: "HYC_ERR_NEGDP"}
HYC_HOST, HYC_DEVICE = 0, 1
NREG_EXTERNAL = -1  # HYC_NREG_EXTERNAL: one block of a decomposed basin (hycadv.decomp)
FIELDS = {"temp": 0, "saln": 1, "th3d": 2, "tracer": 3, "uflx": 4, "vflx": 5, "dp": 6, "oneta": 7, "q2": 8,
          "q2l": 9, "dpo": 10, "onetao": 11, "pbavg": 12, "pbot": 13, "otemp": 14, "osaln": 15, "oth3d": 16,
          "otracer": 17, "oq2": 18, "oq2l": 19, "u": 20, "v": 21, "dpu": 22, "dpv": 23, "ubavg": 24, "vbavg": 25,
          "p": 26, "uflxav": 27, "vflxav": 28, "dpav": 29, "onetacnt": 30}

# every symbol the header declares (checked by the CPU tests)
EXPORTS = ("hyc_bigrid", "hyc_adv_init", "hyc_adv_finalize", "hyc_last_error", "hyc_set_stream", "hyc_bind_field",
           "hyc_sync_field", "hyc_synchronize", "hyc_tsadvc", "hyc_advem", "hyc_xctilr", "hyc_mass_sum",
           "hyc_version", "hyc_enable_timers", "hyc_set_conserve", "hyc_get_stats", "hyc_advem_noalloc", "hyc_ens_create",
           "hyc_ens_destroy", "hyc_ens_set_stream", "hyc_ens_put", "hyc_ens_get",
           "hyc_ens_put_slices", "hyc_ens_get_slices", "hyc_ens_set_tile",
           "hyc_ens_tune", "hyc_ens_step", "hyc_ens_content", "hyc_ens_stats", "hyc_ens_enable_timers",
           "hyc_ens_last_error", "hyc_ens_set_option", "hyc_ens_get_option", "hyc_ens_set_posdef",
           "hyc_za_read", "hyc_za_parse_b", "hyc_za_check", "hyc_set_diffusion_grid", "hyc_tsdff",
           "hyc_asselin_save", "hyc_asselin_filter", "hyc_ens_get_async", "hyc_ens_wait",
           "hyc_set_cnuity_grid", "hyc_cnuity", "hyc_selftest_wait", "hyc_ens_set_diffusion")
ENS_WHAT = {"old": 0, "cur": 1, "uflx": 2, "vflx": 3, "dp": 4}
PRECISION = {"fp64": 0, "mixed": 1}
TIMERS = {"tsadvc": 0, "xctilr": 1, "advect": 2, "copy": 3, "diag": 4, "tsdff": 5, "asselin": 6, "cnuity": 7}


class HycError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Stats(C.Structure):
    _fields_ = [("launches", C.c_int64), ("calls", C.c_int64 * 8), ("ms", C.c_double * 8)]


class BasinSpec(C.Structure):
    _fields_ = [("idm", C.c_int32), ("jdm", C.c_int32), ("kdm", C.c_int32), ("nbdy", C.c_int32),
                ("nreg", C.c_int32), ("ntr", C.c_int32), ("ip", C.POINTER(C.c_int32)),
                ("iu", C.POINTER(C.c_int32)), ("iv", C.POINTER(C.c_int32)), ("scp2", C.POINTER(C.c_double)),
                ("scp2i", C.POINTER(C.c_double))]


class CnuityParams(C.Structure):
    _fields_ = [("nstep", C.c_int32), ("btrmas", C.c_int32), ("thkdf", C.c_int32), ("isopyc", C.c_int32),
                ("delt1", C.c_double), ("ra2fac", C.c_double)]


class TsadvcParams(C.Structure):
    _fields_ = [("advtyp", C.c_int32), ("advflg", C.c_int32), ("btrmas", C.c_int32), ("ntracr", C.c_int32),
                ("nhybrd", C.c_int32), ("isopyc", C.c_int32), ("hybrid", C.c_int32), ("mxlmy", C.c_int32),
                ("nstep", C.c_int32), ("diagno", C.c_int32), ("delt1", C.c_double),
                ("trcflg", C.POINTER(C.c_int32))]


_lib = None


def lib() -> C.CDLL:
    """Load libhycadv.so; raise if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise HycError(-5, f"{LIB_PATH} is missing: build it with __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int32)
        L.hyc_version.restype = C.c_char_p
        L.hyc_bigrid.argtypes = [C.c_int32, C.c_int32, C.c_int32, dp] + [ip] * 8 + [ip]
        L.hyc_adv_init.argtypes = [C.POINTER(vp), C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, ip, ip, ip,
                                   dp, dp, C.c_int32]
        L.hyc_adv_finalize.argtypes = [vp]
        L.hyc_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
        L.hyc_set_stream.argtypes = [vp, vp]
        L.hyc_bind_field.argtypes = [vp, C.c_int32, vp, C.c_int64, C.c_int32]
        L.hyc_sync_field.argtypes = [vp, C.c_int32, C.c_int32]
        L.hyc_synchronize.argtypes = [vp]
        L.hyc_tsadvc.argtypes = [vp, C.c_int32, C.c_int32, C.POINTER(TsadvcParams), dp, dp]
        L.hyc_advem.argtypes = [vp, C.c_int32, vp, vp, vp, vp, vp, vp, C.c_double, vp, vp, C.c_double, C.c_int32,
                                C.c_int32]
        L.hyc_xctilr.argtypes = [vp, vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32]
        L.hyc_mass_sum.argtypes = [vp, vp, vp, dp]
        L.hyc_set_diffusion_grid.argtypes = [vp, dp, dp, dp, dp]
        L.hyc_set_cnuity_grid.argtypes = [vp, dp, dp, dp, dp, dp, dp]
        L.hyc_cnuity.argtypes = [vp, C.c_int32, C.c_int32, C.POINTER(CnuityParams), dp]
        L.hyc_asselin_save.argtypes = [vp, C.c_int32, C.c_int32, C.POINTER(TsadvcParams), C.c_double]
        L.hyc_asselin_filter.argtypes = [vp, C.c_int32, C.c_int32, C.POINTER(TsadvcParams), C.c_double,
                                         C.c_double, C.c_double]
        L.hyc_tsdff.argtypes = [vp, C.c_int32, C.c_int32, C.POINTER(TsadvcParams), C.c_double, C.c_double,
                                C.c_double]
        L.hyc_enable_timers.argtypes = [vp, C.c_int32]
        L.hyc_set_conserve.argtypes = [vp, C.c_int32]
        L.hyc_get_stats.argtypes = [vp, C.POINTER(Stats), C.c_int32]
        L.hyc_ens_create.argtypes = [C.POINTER(vp), C.c_int32, C.POINTER(BasinSpec), C.c_int32, C.c_int32]
        L.hyc_ens_destroy.argtypes = [vp]
        L.hyc_ens_set_stream.argtypes = [vp, vp]
        L.hyc_ens_put.argtypes = [vp, C.c_int32, C.c_int32, vp, C.c_int32]
        L.hyc_ens_get.argtypes = [vp, C.c_int32, C.c_int32, vp, C.c_int32]
        L.hyc_ens_get_async.argtypes = [vp, C.c_int32, C.c_int32, vp, C.c_int32]
        L.hyc_ens_wait.argtypes = [vp]
        L.hyc_selftest_wait.argtypes = [C.c_int32, C.c_int32, C.POINTER(C.c_int32)]
        L.hyc_ens_put_slices.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32, vp, C.c_int32]
        L.hyc_ens_get_slices.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32, vp, C.c_int32]
        L.hyc_ens_set_tile.argtypes = [vp, C.c_int32, C.c_int32]
        L.hyc_ens_tune.argtypes = [vp, C.c_int32, C.c_double, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                   C.POINTER(C.c_double)]
        L.hyc_ens_step.argtypes = [vp, C.c_int32, C.c_double, C.c_int32, C.c_int32]
        L.hyc_ens_content.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.POINTER(C.c_double)]
        L.hyc_ens_stats.argtypes = [vp, C.POINTER(Stats), C.c_int32]
        L.hyc_ens_enable_timers.argtypes = [vp, C.c_int32]
        L.hyc_ens_set_option.argtypes = [vp, C.c_int32, C.c_int32]
        L.hyc_ens_get_option.argtypes = [vp, C.c_int32, C.POINTER(C.c_int32)]
        L.hyc_ens_set_posdef.argtypes = [vp, C.c_int32, C.c_int32, C.c_double]
        L.hyc_ens_set_diffusion.argtypes = [vp, C.c_int32, C.c_double, vp, vp, vp, vp, C.c_int32]
        L.hyc_za_read.argtypes = [C.c_char_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, ip, vp, C.c_int32, dp, dp]
        L.hyc_za_parse_b.argtypes = [C.c_char_p, C.c_char_p, ip, ip, dp, dp]
        L.hyc_za_check.argtypes = [C.c_double] * 4
        L.hyc_ens_last_error.argtypes = [vp]
        L.hyc_ens_last_error.restype = C.c_char_p
        L.hyc_advem_noalloc.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_int32, vp, vp, vp, vp, vp, vp,
                                        C.c_double, vp, vp, C.c_double, vp, vp, vp, vp]
        _lib = L
    return _lib


def version() -> str:
    return lib().hyc_version().decode()


def selftest_wait(arrive: bool, device: int = 0) -> int:
    """hyc_selftest_wait: 1 when a bounded device wait on a barrier nothing
    completes gave up and reported it, 0 when the barrier completed."""
    out = C.c_int32(-1)
    _check(lib().hyc_selftest_wait(int(device), int(bool(arrive)), C.byref(out)))
    return out.value


def _err(h=None) -> str:
    buf = C.create_string_buffer(512)
    lib().hyc_last_error(h, buf, 512)
    return buf.value.decode(errors="replace")


def _check(rc: int, h=None):
    if rc != HYC_OK:
        raise HycError(rc, _err(h))


def _i32(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(C.POINTER(C.c_int32))


def _f64(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(C.POINTER(C.c_double))


def _ptr(a):
    """(pointer, where) of a numpy array (host) or a torch CUDA tensor (device)."""
    if a is None:
        return None, HYC_HOST
    if isinstance(a, np.ndarray):
        if not (a.flags["C_CONTIGUOUS"] and a.dtype == np.float64):
            raise HycError(-1, "host arrays must be C-contiguous float64")
        return a.ctypes.data, HYC_HOST
    import torch

    if isinstance(a, torch.Tensor):
        if not (a.is_contiguous() and a.dtype == torch.float64):
            raise HycError(-1, "tensors must be contiguous float64")
        return a.data_ptr(), (HYC_DEVICE if a.is_cuda else HYC_HOST)
    raise TypeError(type(a))


class _StreamFollower:
    """Stream ordering between torch and the library.

    The library queues its work on one CUDA stream per context (its own
    non-blocking stream unless set_stream chose another).  Device tensors
    handed over from torch were written on torch's current stream, so by
    default the wrappers put the library on torch's current stream of the
    device before each call that queues work: reads of torch-produced
    tensors and torch's later reads of the library's results are then
    ordered by the stream itself.  After an explicit set_stream the caller
    owns the ordering, and the wrappers wait for torch's current stream
    before a call that passes it device tensors."""

    def _init_stream(self, device: int):
        self.device = device
        self._explicit = None  # stream pointer chosen by set_stream
        self._cur = None       # stream pointer the library uses now (None: its own)

    def _set_stream_ptr(self, ptr: int):
        raise NotImplementedError

    def _order(self, tensors=()):
        import sys

        torch = sys.modules.get("torch")
        if torch is None or not torch.cuda.is_available():
            return
        cur = torch.cuda.current_stream(self.device)
        if self._explicit is None:
            if self._cur != cur.cuda_stream:
                self._set_stream_ptr(cur.cuda_stream)
                self._cur = cur.cuda_stream
        elif cur.cuda_stream != self._explicit and any(
                isinstance(t, torch.Tensor) and t.is_cuda for t in tensors):
            cur.synchronize()


def bigrid(depth: np.ndarray, nbdy: int = 6):
    """bigrid.F90 for one tile: returns (depth_after, masks, nreg).

    masks has ip, iu, iv, iq, ipim1, ipip1, ipjm1, ipjp1 (int32, (ld2, ld1)).
    """
    d, dptr = _f64(np.array(depth, dtype=np.float64, copy=True))
    ld2, ld1 = d.shape
    idm, jdm = ld1 - 2 * nbdy, ld2 - 2 * nbdy
    names = ("ip", "iu", "iv", "iq", "ipim1", "ipip1", "ipjm1", "ipjp1")
    masks = {k: np.zeros((ld2, ld1), np.int32) for k in names}
    nreg = C.c_int32(-1)
    _check(lib().hyc_bigrid(idm, jdm, nbdy, dptr, *[_i32(masks[k])[1] for k in names], C.byref(nreg)))
    return d, masks, nreg.value


class Context(_StreamFollower):
    """One basin on one GPU: the state tsadvc reads from mod_dimensions/mod_cb_arrays."""

    def __init__(self, idm, jdm, kdm, nbdy, nreg, ip, iu, iv, scp2, scp2i, device: int = 0):
        L = lib()
        self.idm, self.jdm, self.kdm, self.nbdy, self.nreg = idm, jdm, kdm, nbdy, nreg
        self.ld1, self.ld2 = idm + 2 * nbdy, jdm + 2 * nbdy
        self.slice = self.ld1 * self.ld2
        h = C.c_void_p()
        keep = [_i32(ip), _i32(iu), _i32(iv), _f64(scp2), _f64(scp2i)]
        _check(L.hyc_adv_init(C.byref(h), idm, jdm, kdm, nbdy, nreg, keep[0][1], keep[1][1], keep[2][1], keep[3][1],
                              keep[4][1], device))
        self._h = h
        self._bound = {}
        self._init_stream(device)

    def _set_stream_ptr(self, ptr: int):
        _check(lib().hyc_set_stream(self._h, C.c_void_p(ptr)), self._h)

    @classmethod
    def from_masks(cls, masks: dict, scp2, scp2i, kdm: int, nreg: int, nbdy: int = 6, device: int = 0):
        ld2, ld1 = masks["ip"].shape
        return cls(ld1 - 2 * nbdy, ld2 - 2 * nbdy, kdm, nbdy, nreg, masks["ip"], masks["iu"], masks["iv"], scp2,
                   scp2i, device)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().hyc_adv_finalize(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- fields -------------------------------------------------------------
    def bind(self, name: str, array):
        """Bind a model field: a torch CUDA tensor is used in place; a numpy
        array gets a resident device mirror (move data with :meth:`sync`)."""
        p, where = _ptr(array)
        n = array.size if isinstance(array, np.ndarray) else array.numel()
        self._order((array,))
        _check(lib().hyc_bind_field(self._h, FIELDS[name], p, n, where), self._h)
        self._bound[name] = array

    def sync(self, name: str, to_device: bool):
        self._order(self._bound.values())
        _check(lib().hyc_sync_field(self._h, FIELDS[name], int(bool(to_device))), self._h)

    def synchronize(self):
        _check(lib().hyc_synchronize(self._h), self._h)

    def set_stream(self, stream):
        """Queue later work on a torch.cuda.Stream (or a raw cudaStream_t int).
        The caller then orders it against torch's other streams."""
        ptr = stream if isinstance(stream, int) else stream.cuda_stream
        self._set_stream_ptr(ptr)
        self._explicit = self._cur = ptr

    # -- the reference's routines --------------------------------------------
    def tsadvc(self, m: int, n: int, *, delt1: float, advtyp: int = 2, advflg: int = 0, btrmas: bool = False,
               ntracr: int = 0, trcflg=None, nhybrd: int | None = None, isopyc: bool = False, mxlmy: bool = False,
               nstep: int = 1, diagno: bool = False, range_diag: bool = False):
        """tsadvc(m,n) on the bound fields.  Returns (xmin, xmax) of salinity
        per layer when range_diag and the diagnostic runs, else None."""
        nh = self.kdm if nhybrd is None else nhybrd
        tf = np.ascontiguousarray(trcflg if trcflg is not None else np.zeros(max(ntracr, 1)), np.int32)
        p = TsadvcParams(advtyp=advtyp, advflg=advflg, btrmas=int(btrmas), ntracr=ntracr, nhybrd=nh,
                         isopyc=int(isopyc), hybrid=int(nh > 0), mxlmy=int(mxlmy), nstep=nstep, diagno=int(diagno),
                         delt1=float(delt1), trcflg=tf.ctypes.data_as(C.POINTER(C.c_int32)))
        self._order(self._bound.values())
        if range_diag and (nstep % 3 == 0 or diagno):  # mod_tsadvc.F90:2065
            xmin = np.zeros(self.kdm)
            xmax = np.zeros(self.kdm)
            _check(lib().hyc_tsadvc(self._h, m, n, C.byref(p), xmin.ctypes.data_as(C.POINTER(C.c_double)),
                                    xmax.ctypes.data_as(C.POINTER(C.c_double))), self._h)
            return xmin, xmax
        _check(lib().hyc_tsadvc(self._h, m, n, C.byref(p), None, None), self._h)
        return None

    def set_diffusion_grid(self, aspux, aspvy, scuy, scvx):
        """Grid arrays of the lateral diffusion (host, ld1*ld2 each)."""
        keep = [_f64(a) for a in (aspux, aspvy, scuy, scvx)]
        _check(lib().hyc_set_diffusion_grid(self._h, *[k[1] for k in keep]), self._h)

    def tsdff(self, m: int, n: int, *, delt1: float, temdf2: float, temdfc: float = 1.0, thbase: float = 34.0,
              ntracr: int = 0, nhybrd: int | None = None, isopyc: bool = False, mxlmy: bool = False):
        """The diffusion block at the end of tsadvc(m,n) on the bound fields
        (level n in place, th3d from the new temp and saln)."""
        nh = self.kdm if nhybrd is None else nhybrd
        tf = np.zeros(max(ntracr, 1), np.int32)
        p = TsadvcParams(advtyp=2, advflg=0, btrmas=0, ntracr=ntracr, nhybrd=nh, isopyc=int(isopyc),
                         hybrid=int(nh > 0), mxlmy=int(mxlmy), nstep=1, diagno=0, delt1=float(delt1),
                         trcflg=tf.ctypes.data_as(C.POINTER(C.c_int32)))
        self._order(self._bound.values())
        _check(lib().hyc_tsdff(self._h, m, n, C.byref(p), float(temdf2), float(temdfc), float(thbase)), self._h)

    def _params(self, ntracr=0, nhybrd=None, advflg=0, isopyc=False, mxlmy=False, delt1=0.0):
        nh = self.kdm if nhybrd is None else nhybrd
        tf = np.zeros(max(ntracr, 1), np.int32)
        p = TsadvcParams(advtyp=2, advflg=advflg, btrmas=0, ntracr=ntracr, nhybrd=nh, isopyc=int(isopyc),
                         hybrid=int(nh > 0), mxlmy=int(mxlmy), nstep=1, diagno=0, delt1=float(delt1),
                         trcflg=tf.ctypes.data_as(C.POINTER(C.c_int32)))
        return p, tf

    def set_cnuity_grid(self, scuy, scvx, depthu, depthv, thkdfu=None, thkdfv=None):
        """Grid arrays of cnuity (host, ld1*ld2 each; thkdf* may be None)."""
        keep = [_f64(a) for a in (scuy, scvx, depthu, depthv)]
        th = [(None, None) if a is None else _f64(a) for a in (thkdfu, thkdfv)]
        _check(lib().hyc_set_cnuity_grid(self._h, *[k[1] for k in keep], th[0][1], th[1][1]), self._h)

    def cnuity(self, m: int, n: int, *, delt1: float, nstep: int = 1, btrmas: bool = False, thkdf: int = 0,
               ra2fac: float = 0.125, want_dpkmin: bool = False):
        """cnuity(m,n) on the bound fields.  Returns dpkmin (2*kdm) when asked."""
        p = CnuityParams(nstep=nstep, btrmas=int(btrmas), thkdf=int(thkdf), isopyc=0, delt1=float(delt1),
                         ra2fac=float(ra2fac))
        out = np.zeros(2 * self.kdm) if want_dpkmin else None
        self._order(self._bound.values())
        _check(lib().hyc_cnuity(self._h, m, n, C.byref(p), None if out is None else
                                out.ctypes.data_as(C.POINTER(C.c_double))), self._h)
        return out

    def asselin_save(self, m: int, n: int, *, oneta0: float, ntracr: int = 0, mxlmy: bool = False):
        """asselin_save(m,n) on the bound fields (start of a step)."""
        p, tf = self._params(ntracr=ntracr, mxlmy=mxlmy)
        self._order(self._bound.values())
        _check(lib().hyc_asselin_save(self._h, m, n, C.byref(p), float(oneta0)), self._h)

    def asselin_filter(self, m: int, n: int, *, ra2fac: float, oneta0: float, thbase: float = 34.0, ntracr: int = 0,
                       mxlmy: bool = False, nhybrd: int | None = None, advflg: int = 0):
        """asselin_filter(m,n) on the bound fields (end of a step)."""
        p, tf = self._params(ntracr=ntracr, nhybrd=nhybrd, advflg=advflg, mxlmy=mxlmy)
        self._order(self._bound.values())
        _check(lib().hyc_asselin_filter(self._h, m, n, C.byref(p), float(ra2fac), float(oneta0), float(thbase)),
               self._h)

    def advem(self, advtyp, fld, fldc, u, v, fco, fcn, posdef, scal, scali, dt2, btrmas=False):
        """advem on one slice; all arrays numpy (host) or all torch CUDA (device)."""
        arrs = [fld, fldc, u, v, fco, fcn, scal, scali]
        ptrs = [_ptr(a) for a in arrs]
        wheres = {w for (p, w), a in zip(ptrs, arrs) if a is not None}
        if len(wheres) != 1:
            raise HycError(-1, "advem arrays must all be host or all device")
        where = wheres.pop()
        p = [pp for pp, _ in ptrs]
        self._order(arrs)
        _check(lib().hyc_advem(self._h, int(advtyp), p[0], p[1], p[2], p[3], p[4], p[5], float(posdef), p[6], p[7],
                               float(dt2), int(bool(btrmas)), where), self._h)

    def xctilr(self, a, mh: int, nh: int):
        p, where = _ptr(a)
        nlev = int(np.prod(a.shape[:-2])) if len(a.shape) > 2 else 1
        self._order((a,))
        _check(lib().hyc_xctilr(self._h, p, nlev, mh, nh, where), self._h)

    def enable_timers(self, on: bool = True):
        _check(lib().hyc_enable_timers(self._h, int(bool(on))), self._h)

    def set_conserve(self, on: bool = True):
        """advem's explicit conservation rescale (mod_tsadvc.F90:32, :168-203)."""
        _check(lib().hyc_set_conserve(self._h, int(bool(on))), self._h)

    def stats(self, reset: bool = False) -> dict:
        """Kernel launches and device-time per timer slot (ms, calls)."""
        s = Stats()
        _check(lib().hyc_get_stats(self._h, C.byref(s), int(bool(reset))), self._h)
        out = {"launches": int(s.launches)}
        for name, i in TIMERS.items():
            out[name] = (float(s.ms[i]), int(s.calls[i]))
        return out

    def mass_sum(self, fld, fc) -> float:
        """sum over interior sea cells of fld*(fc+onemu)*scp2 (device tensors)."""
        out = C.c_double(0.0)
        self._order((fld, fc))
        _check(lib().hyc_mass_sum(self._h, _ptr(fld)[0], _ptr(fc)[0], C.byref(out)), self._h)
        return out.value


class Ensemble(_StreamFollower):
    """Many independent basins advected together (hyc_ens_* in the C ABI).

    basins: list of dicts with idm, jdm, kdm, nbdy, nreg, ntr and the
    bigrid masks ip/iu/iv plus scp2/scp2i (numpy, reference layout).
    precision: "fp64" (plain form) or "mixed" (FP32-mixed form).
    """

    def __init__(self, basins, precision: str = "fp64", device: int = 0):
        L = lib()
        self._keep = []
        specs = (BasinSpec * len(basins))()
        for i, b in enumerate(basins):
            ip, iu, iv = _i32(b["ip"]), _i32(b["iu"]), _i32(b["iv"])
            sc, si = _f64(b["scp2"]), _f64(b["scp2i"])
            self._keep += [ip, iu, iv, sc, si]
            specs[i] = BasinSpec(b["idm"], b["jdm"], b["kdm"], b["nbdy"], b["nreg"], b["ntr"], ip[1], iu[1], iv[1],
                                 sc[1], si[1])
        h = C.c_void_p()
        _check(L.hyc_ens_create(C.byref(h), len(basins), specs, PRECISION[precision], device))
        self._h = h
        self.basins = [dict(b) for b in basins]
        self.precision = precision
        self._init_stream(device)

    def _set_stream_ptr(self, ptr: int):
        self._chk(lib().hyc_ens_set_stream(self._h, C.c_void_p(ptr)))

    def _chk(self, rc):
        if rc != HYC_OK:
            raise HycError(rc, lib().hyc_ens_last_error(self._h).decode(errors="replace"))

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().hyc_ens_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream):
        """Queue later work on a torch.cuda.Stream (or a raw cudaStream_t int);
        graphs are replayed there.  The caller then orders it against
        torch's other streams."""
        ptr = stream if isinstance(stream, int) else stream.cuda_stream
        self._set_stream_ptr(ptr)
        self._explicit = self._cur = ptr

    def put(self, b: int, what: str, a, s0: int = None, ns: int = None):
        """Whole field, or (s0, ns) the slices [s0, s0+ns) only (tracer q of
        old/cur is s0 = q*kdm, ns = kdm)."""
        p, where = _ptr(a)
        self._order((a,))
        if s0 is None:
            self._chk(lib().hyc_ens_put(self._h, b, ENS_WHAT[what], p, where))
        else:
            self._chk(lib().hyc_ens_put_slices(self._h, b, ENS_WHAT[what], s0, ns, p, where))

    def get(self, b: int, what: str, out, s0: int = None, ns: int = None):
        p, where = _ptr(out)
        self._order((out,))
        if s0 is None:
            self._chk(lib().hyc_ens_get(self._h, b, ENS_WHAT[what], p, where))
        else:
            self._chk(lib().hyc_ens_get_slices(self._h, b, ENS_WHAT[what], s0, ns, p, where))
        return out

    def get_async(self, b: int, what: str, out):
        """hyc_ens_get_async: the copy into out overlaps later work; call
        wait() before reading out."""
        p, where = _ptr(out)
        self._order((out,))
        self._chk(lib().hyc_ens_get_async(self._h, b, ENS_WHAT[what], p, where))
        return out

    def wait(self):
        self._chk(lib().hyc_ens_wait(self._h))

    def set_tile(self, tx: int, ty: int):
        self._chk(lib().hyc_ens_set_tile(self._h, tx, ty))

    def tune(self, advtyp: int, delt1: float):
        tx, ty, ms = C.c_int32(), C.c_int32(), C.c_double()
        self._order()
        self._chk(lib().hyc_ens_tune(self._h, advtyp, float(delt1), C.byref(tx), C.byref(ty), C.byref(ms)))
        return tx.value, ty.value, ms.value

    def step(self, advtyp: int, delt1: float, nsteps: int = 1, graph: bool = False):
        self._order()
        self._chk(lib().hyc_ens_step(self._h, advtyp, float(delt1), nsteps, int(bool(graph))))

    def content(self, b: int, q: int, what: str, delt1: float) -> float:
        out = C.c_double()
        self._order()
        self._chk(lib().hyc_ens_content(self._h, b, q, ENS_WHAT[what], float(delt1), C.byref(out)))
        return out.value

    def enable_timers(self, on: bool = True):
        self._chk(lib().hyc_ens_enable_timers(self._h, int(bool(on))))

    def set_prep64(self, on: bool):
        """Mixed form: thickness prep in FP64 (True, default) or compensated FP32."""
        self._chk(lib().hyc_ens_set_option(self._h, 1, int(bool(on))))

    def set_posdef(self, b: int, q: int, posdef: float):
        """MPDATA offset of tracer q of basin b (mod_tsadvc.F90:1755-1763)."""
        self._chk(lib().hyc_ens_set_posdef(self._h, b, q, float(posdef)))

    def set_diffusion(self, b: int, temdf2: float, aspux=None, aspvy=None, scuy=None, scvx=None):
        """Lateral diffusion of basin b's tracers after each step, fused into
        the mixed form's step kernel (hyc_ens_set_diffusion); grid arrays in
        the reference layout (numpy or CUDA tensors, all on the same side);
        temdf2 = 0 turns it off."""
        if temdf2 > 0:
            arrs = [aspux, aspvy, scuy, scvx]
            ptrs = [_ptr(a) for a in arrs]
            if len({w for _, w in ptrs}) != 1:
                raise ValueError("grid arrays must all be on the host or all on the device")
            self._order(tuple(a for a in arrs if not isinstance(a, np.ndarray)))
            self._chk(lib().hyc_ens_set_diffusion(self._h, b, float(temdf2), *[p for p, _ in ptrs], ptrs[0][1]))
        else:  # 0 turns it off; a negative value is refused by the library
            self._chk(lib().hyc_ens_set_diffusion(self._h, b, float(temdf2), None, None, None, None, HYC_HOST))

    def set_strip_tracers(self, n: int):
        """Mixed form: tracers advanced per pass of the strip kernel (1 or 2)."""
        self._chk(lib().hyc_ens_set_option(self._h, 3, int(n)))

    def option(self, name: str) -> int:
        """Current value of an option: "prep64" or "strip_tracers"."""
        v = C.c_int32()
        self._chk(lib().hyc_ens_get_option(self._h, {"prep64": 1, "strip_tracers": 3}[name], C.byref(v)))
        return v.value

    def stats(self, reset: bool = False) -> dict:
        s = Stats()
        self._chk(lib().hyc_ens_stats(self._h, C.byref(s), int(bool(reset))))
        return {"launches": int(s.launches), "step_ms": float(s.ms[2]), "step_calls": int(s.calls[2]),
                "copy_ms": float(s.ms[3]), "copy_calls": int(s.calls[3]), "stage_kernels_ms": float(s.ms[1])}
