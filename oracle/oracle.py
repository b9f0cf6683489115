"""ctypes front end of the CPU oracle (oracle/hyc_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
benchmark's CPU-baseline leg.  The product path never imports it.

Arrays follow the reference layout (see hyc_oracle.c): numpy float64 / int32,
C-contiguous, a 2-D slice has shape (ld2, ld1) = (jdm+2*nbdy, idm+2*nbdy).
Parity unpinned: there are no reference golden vectors for this path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libhyc_oracle.so")
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (see oracle/Makefile)."""
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
            os.path.join(_HERE, "hyc_oracle.c")):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int32)
        L.hyo_grid_create.restype = C.c_void_p
        L.hyo_grid_create.argtypes = [C.c_int, C.c_int, C.c_int, dp, dp, dp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.hyo_grid_from_masks.restype = C.c_void_p
        L.hyo_grid_from_masks.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, ip, ip, ip, dp, dp, C.POINTER(C.c_int)]
        L.hyo_grid_free.argtypes = [C.c_void_p]
        L.hyo_grid_nreg.argtypes = [C.c_void_p]
        L.hyo_grid_masks.argtypes = [C.c_void_p] + [ip] * 7
        L.hyo_grid_work.argtypes = [C.c_void_p, C.c_char_p, dp]
        L.hyo_set_threads.argtypes = [C.c_void_p, C.c_int]
        L.hyo_set_conserve.argtypes = [C.c_void_p, C.c_int]
        L.hyo_max_threads.restype = C.c_int
        L.hyo_xctilr.argtypes = [C.c_void_p, dp, C.c_int, C.c_int, C.c_int]
        L.hyo_advem.argtypes = [C.c_void_p, C.c_int, dp, dp, dp, dp, dp, dp, C.c_double, dp, dp, C.c_double, C.c_int]
        L.hyo_tsadvc.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int] + [dp] * 12
        L.hyo_tsdff.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int] + [dp] * 12
        L.hyo_asselin_save.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_void_p]
        L.hyo_asselin_filter.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_int,
                                         C.c_int, C.c_void_p]
        L.hyo_cnuity.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, dp]
        L.hyo_sig.restype = C.c_double
        L.hyo_sig.argtypes = [C.c_double, C.c_double]
        L.hyo_xcsum.restype = C.c_double
        L.hyo_xcsum.argtypes = [C.c_void_p, dp, ip]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "oracle arrays must be C-contiguous"
    if a.dtype == np.float64:
        return a.ctypes.data_as(C.POINTER(C.c_double))
    if a.dtype == np.int32:
        return a.ctypes.data_as(C.POINTER(C.c_int32))
    raise TypeError(a.dtype)


class _TsParams(C.Structure):
    _fields_ = [("kdm", C.c_int), ("advtyp", C.c_int), ("advflg", C.c_int), ("btrmas", C.c_int),
                ("ntracr", C.c_int), ("nhybrd", C.c_int), ("isopyc", C.c_int), ("hybrid", C.c_int),
                ("mxlmy", C.c_int), ("nstep", C.c_int), ("diagno", C.c_int), ("delt1", C.c_double),
                ("trcflg", C.POINTER(C.c_int32))]


class OracleError(RuntimeError):
    pass


class Grid:
    """bigrid + the module work arrays of mod_tsadvc for one basin."""

    def __init__(self, depth: np.ndarray, scp2: np.ndarray, scp2i: np.ndarray, nbdy: int = 6,
                 threads: int = 0):
        L = lib()
        self.nbdy = nbdy
        self.ld2, self.ld1 = depth.shape
        self.idm = self.ld1 - 2 * nbdy
        self.jdm = self.ld2 - 2 * nbdy
        self.depth = np.ascontiguousarray(depth, dtype=np.float64).copy()
        err = C.c_int(0)
        nfill = C.c_int(0)
        h = L.hyo_grid_create(self.idm, self.jdm, nbdy, _p(self.depth),
                              _p(np.ascontiguousarray(scp2, np.float64)),
                              _p(np.ascontiguousarray(scp2i, np.float64)), C.byref(err), C.byref(nfill))
        if not h:
            raise OracleError(f"hyo_grid_create failed: err={err.value} one-point seas={nfill.value}")
        self._h = C.c_void_p(h)
        self.scp2 = np.ascontiguousarray(scp2, np.float64)
        self.scp2i = np.ascontiguousarray(scp2i, np.float64)
        self.nreg = L.hyo_grid_nreg(self._h)
        shp = (self.ld2, self.ld1)
        m = {k: np.zeros(shp, np.int32) for k in ("ip", "iu", "iv", "ipim1", "ipip1", "ipjm1", "ipjp1")}
        L.hyo_grid_masks(self._h, *[_p(m[k]) for k in ("ip", "iu", "iv", "ipim1", "ipip1", "ipjm1", "ipjp1")])
        self.masks = m
        if threads:
            self.set_threads(threads)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib is not None:
            _lib.hyo_grid_free(h)
            self._h = None

    @classmethod
    def from_masks(cls, ip, iu, iv, scp2, scp2i, nbdy: int = 6, nreg: int = -1, threads: int = 0):
        """A tile of a decomposed basin: its window (with halo) of the basin's
        masks and metrics.  nreg < 0: halos come from the caller's exchange."""
        L = lib()
        self = cls.__new__(cls)
        self.nbdy = nbdy
        self.ld2, self.ld1 = ip.shape
        self.idm = self.ld1 - 2 * nbdy
        self.jdm = self.ld2 - 2 * nbdy
        self.depth = None
        keep = [np.ascontiguousarray(a, np.int32) for a in (ip, iu, iv)]
        self.scp2 = np.ascontiguousarray(scp2, np.float64)
        self.scp2i = np.ascontiguousarray(scp2i, np.float64)
        err = C.c_int(0)
        h = L.hyo_grid_from_masks(self.idm, self.jdm, nbdy, nreg, *[_p(k) for k in keep], _p(self.scp2),
                                  _p(self.scp2i), C.byref(err))
        if not h:
            raise OracleError(f"hyo_grid_from_masks failed: err={err.value}")
        self._h = C.c_void_p(h)
        self.nreg = nreg
        shp = (self.ld2, self.ld1)
        m = {k: np.zeros(shp, np.int32) for k in ("ip", "iu", "iv", "ipim1", "ipip1", "ipjm1", "ipjp1")}
        L.hyo_grid_masks(self._h, *[_p(m[k]) for k in ("ip", "iu", "iv", "ipim1", "ipip1", "ipjm1", "ipjp1")])
        self.masks = m
        if threads:
            self.set_threads(threads)
        return self

    def set_threads(self, n: int):
        lib().hyo_set_threads(self._h, int(n))

    def set_conserve(self, on: bool):
        """advem's explicit conservation rescale (mod_tsadvc.F90:32, :168-203)."""
        lib().hyo_set_conserve(self._h, int(bool(on)))

    def xctilr(self, a: np.ndarray, mh: int, nh: int):
        nlev = int(np.prod(a.shape[:-2])) if a.ndim > 2 else 1
        lib().hyo_xctilr(self._h, _p(a), nlev, mh, nh)

    def advem(self, advtyp, fld, fldc, u, v, fco, fcn, posdef, scal, scali, dt2, btrmas=False):
        rc = lib().hyo_advem(self._h, int(advtyp), _p(fld), _p(fldc), _p(u), _p(v), _p(fco), _p(fcn),
                             float(posdef), _p(scal), _p(scali), float(dt2), int(bool(btrmas)))
        if rc != 0:
            raise OracleError(f"advem rc={rc}")

    def work(self, name: str) -> np.ndarray:
        out = np.empty((self.ld2, self.ld1), np.float64)
        if lib().hyo_grid_work(self._h, name.encode(), _p(out)) != 0:
            raise KeyError(name)
        return out

    def xcsum(self, a: np.ndarray, mask: np.ndarray) -> float:
        return lib().hyo_xcsum(self._h, _p(a), _p(np.ascontiguousarray(mask, np.int32)))

    def tsadvc(self, m: int, n: int, *, temp, saln, th3d, uflx, vflx, dp, delt1, advtyp=2, advflg=0,
               btrmas=False, tracer=None, trcflg=None, nhybrd=None, isopyc=False, mxlmy=False, q2=None,
               q2l=None, oneta=None, nstep=1, diagno=False):
        kdm = temp.shape[1]
        ntr = 0 if tracer is None else tracer.shape[0]
        tf = np.ascontiguousarray(trcflg if trcflg is not None else np.zeros(max(ntr, 1)), np.int32)
        p = _TsParams(kdm=kdm, advtyp=advtyp, advflg=advflg, btrmas=int(btrmas), ntracr=ntr,
                      nhybrd=kdm if nhybrd is None else nhybrd, isopyc=int(isopyc),
                      hybrid=int((kdm if nhybrd is None else nhybrd) > 0), mxlmy=int(mxlmy), nstep=nstep,
                      diagno=int(diagno), delt1=float(delt1), trcflg=_p(tf))
        xmin = np.zeros(kdm)
        xmax = np.zeros(kdm)
        rc = lib().hyo_tsadvc(self._h, C.byref(p), m, n, _p(temp), _p(saln), _p(th3d), _p(tracer), _p(uflx),
                              _p(vflx), _p(dp), _p(oneta), _p(q2), _p(q2l), _p(xmin), _p(xmax))
        if rc != 0:
            raise OracleError(f"tsadvc rc={rc}")
        return xmin, xmax

    def _assel_params(self, kdm, ntracr, mxlmy, nhybrd=None, advflg=0, isopyc=False):
        tf = np.zeros(max(ntracr, 1), np.int32)
        p = _TsParams(kdm=kdm, advtyp=2, advflg=advflg, btrmas=0, ntracr=ntracr,
                      nhybrd=kdm if nhybrd is None else nhybrd, isopyc=int(isopyc), hybrid=1, mxlmy=int(mxlmy),
                      nstep=1, diagno=0, delt1=0.0, trcflg=_p(tf))
        return p, tf

    def asselin_save(self, m: int, n: int, arrays: dict, *, oneta0: float):
        """asselin_save(m,n) (mod_asselin.F90:28-82) on the arrays named as in
        ASSELIN_ARRAYS (numpy, reference layout)."""
        kdm = arrays["temp"].shape[1]
        ntr = 0 if arrays.get("tracer") is None else arrays["tracer"].shape[0]
        p, tf = self._assel_params(kdm, ntr, arrays.get("q2") is not None)
        rc = lib().hyo_asselin_save(self._h, C.byref(p), float(oneta0), m, n, _assel_ptrs(arrays))
        if rc != 0:
            raise OracleError(f"asselin_save rc={rc}")

    def asselin_filter(self, m: int, n: int, arrays: dict, *, ra2fac: float, oneta0: float, thbase: float = 34.0,
                       nhybrd=None, advflg=0):
        """asselin_filter(m,n) (mod_asselin.F90:84-268), advflg=0 hybrid layers."""
        kdm = arrays["temp"].shape[1]
        ntr = 0 if arrays.get("tracer") is None else arrays["tracer"].shape[0]
        p, tf = self._assel_params(kdm, ntr, arrays.get("q2") is not None, nhybrd, advflg)
        rc = lib().hyo_asselin_filter(self._h, C.byref(p), float(ra2fac), float(oneta0), float(thbase), m, n,
                                      _assel_ptrs(arrays))
        if rc != 0:
            raise OracleError(f"asselin_filter rc={rc}")

    def cnuity(self, m: int, n: int, arrays: dict, *, delt1: float, nstep: int = 1, btrmas: bool = False,
               thkdf4: bool = False, thkdf2: bool = False, ra2fac: float = 0.125):
        """cnuity(m,n) (cnuity.F90) on the arrays named as in CNUITY_ARRAYS
        (numpy, reference layout; inputs' halos are refreshed in place).
        Returns dpkmin (2*kdm: after the low-order and the antidiffusive
        update of each layer); raises OracleError(-9) on a fatal negative
        thickness (checked when nstep % 3 == 0)."""
        kdm = arrays["dp"].shape[1]
        for k, v in arrays.items():
            if k not in CNUITY_ARRAYS:
                raise KeyError(k)
            if v is not None and not (v.flags["C_CONTIGUOUS"] and v.dtype == np.float64):
                raise OracleError(f"{k}: need C-contiguous float64")
        ptrs = (C.c_void_p * len(CNUITY_ARRAYS))()
        for i, k in enumerate(CNUITY_ARRAYS):
            v = arrays.get(k)
            ptrs[i] = None if v is None else v.ctypes.data
        p = _CnParams(kdm=kdm, nstep=nstep, btrmas=int(btrmas), thkdf4=int(thkdf4), thkdf2=int(thkdf2),
                      delt1=float(delt1), ra2fac=float(ra2fac))
        dpkmin = np.zeros(2 * kdm)
        rc = lib().hyo_cnuity(self._h, C.byref(p), m, n, ptrs, _p(dpkmin))
        if rc != 0:
            err = OracleError(f"cnuity rc={rc}")
            err.code = rc
            raise err
        return dpkmin

    def tsdff(self, m: int, n: int, *, temp, saln, th3d, dp, oneta, aspux, aspvy, scuy, scvx, delt1, temdf2,
              temdfc=1.0, thbase=34.0, tracer=None, q2=None, q2l=None, advflg=0, nhybrd=None, isopyc=False):
        """The diffusion block of tsadvc(m,n) (mod_tsadvc.F90:2138-2230),
        in place on level n; q2/q2l (2, kdm+2, ld2, ld1) given = mxlmy."""
        mxlmy = q2 is not None
        kdm = temp.shape[1]
        ntr = 0 if tracer is None else tracer.shape[0]
        tf = np.zeros(max(ntr, 1), np.int32)
        p = _TsParams(kdm=kdm, advtyp=2, advflg=advflg, btrmas=0, ntracr=ntr,
                      nhybrd=kdm if nhybrd is None else nhybrd, isopyc=int(isopyc), hybrid=1, mxlmy=int(mxlmy),
                      nstep=1, diagno=0, delt1=float(delt1), trcflg=_p(tf))
        rc = lib().hyo_tsdff(self._h, C.byref(p), float(temdf2), float(temdfc), float(thbase), m, n, _p(temp),
                             _p(saln), _p(th3d), _p(tracer), _p(q2), _p(q2l), _p(dp), _p(oneta), _p(aspux), _p(aspvy), _p(scuy),
                             _p(scvx))
        if rc != 0:
            raise OracleError(f"tsdff rc={rc}")


ASSELIN_ARRAYS = ("temp", "saln", "th3d", "tracer", "q2", "q2l", "dp", "dpo", "oneta", "onetao", "pbavg", "pbot",
                  "otemp", "osaln", "oth3d", "otracer", "oq2", "oq2l")


def _assel_ptrs(arrs: dict):
    for k, v in arrs.items():
        if k not in ASSELIN_ARRAYS:
            raise KeyError(k)
        if v is not None and not (v.flags["C_CONTIGUOUS"] and v.dtype == np.float64):
            raise OracleError(f"{k}: need C-contiguous float64")
    ptrs = (C.c_void_p * len(ASSELIN_ARRAYS))()
    for i, k in enumerate(ASSELIN_ARRAYS):
        v = arrs.get(k)
        ptrs[i] = None if v is None else v.ctypes.data
    return ptrs


CNUITY_ARRAYS = ("dp", "dpo", "dpu", "dpv", "u", "v", "ubavg", "vbavg", "pbot", "depthu", "depthv", "oneta", "scuy",
                 "scvx", "thkdfu", "thkdfv", "p", "uflx", "vflx", "uflxav", "vflxav", "dpav", "onetacnt")
ERR_NEGDP = -9


class _CnParams(C.Structure):
    _fields_ = [("kdm", C.c_int), ("nstep", C.c_int), ("btrmas", C.c_int), ("thkdf4", C.c_int), ("thkdf2", C.c_int),
                ("delt1", C.c_double), ("ra2fac", C.c_double)]


def sig(t: float, s: float) -> float:
    """sigma-2 of the 17-term equation of state (stmt_fns.h:497-505)."""
    return lib().hyo_sig(float(t), float(s))


def max_threads() -> int:
    return lib().hyo_max_threads()
