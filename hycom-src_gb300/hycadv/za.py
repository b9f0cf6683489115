"""HYCOM .a/.b field input over the C ABI (hyc_za_*): read fields of a
HYCOM restart or archive file into reference-layout arrays, as
zaiord/restart_in3d do (mod_za_sm.h:700-780, mod_restart.F90:561-620)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import HycError, _check, _ptr, lib


def read_record(path: str, record: int, idm: int, jdm: int, nbdy: int, out, mask=None):
    """Record (1-based) of a .a file into the interior of `out`, a numpy or
    torch (CPU or CUDA) float64 array in the reference layout (jdm+2*nbdy,
    idm+2*nbdy).  mask: int32 array of the same layout or None.  Returns
    (hmin, hmax)."""
    p, where = _ptr(out)
    m = None
    if mask is not None:
        mask = np.ascontiguousarray(mask, dtype=np.int32)
        m = mask.ctypes.data_as(C.POINTER(C.c_int32))
    lo, hi = C.c_double(), C.c_double()
    _check(lib().hyc_za_read(path.encode(), idm, jdm, nbdy, record, m, p, where, C.byref(lo), C.byref(hi)))
    return lo.value, hi.value


def parse_b(line: str):
    """(cfield, layer, level, hmin, hmax) of one .b line."""
    cf = C.create_string_buffer(9)
    lay, lev = C.c_int32(), C.c_int32()
    lo, hi = C.c_double(), C.c_double()
    _check(lib().hyc_za_parse_b(line.encode(), cf, C.byref(lay), C.byref(lev), C.byref(lo), C.byref(hi)))
    return cf.value.decode(), lay.value, lev.value, lo.value, hi.value


def restart_index(bpath: str, header_lines: int = 2):
    """Records of a restart .b file: {(cfield stripped, layer, level):
    (record, hmin, hmax)}; record i is the i-th line after the header."""
    out = {}
    with open(bpath) as f:
        lines = f.read().splitlines()[header_lines:]
    for r, ln in enumerate(lines, start=1):
        if "=" not in ln:
            continue
        cf, lay, lev, lo, hi = parse_b(ln)
        out[(cf.strip(), lay, lev)] = (r, lo, hi)
    return out


def read_restart_field(apath: str, bpath: str, name: str, layer: int, level: int, idm: int, jdm: int, nbdy: int,
                       out, header_lines: int = 2):
    """One field of a restart file pair, checked against its .b range as
    restart_in3d does (1e-4 relative)."""
    idx = restart_index(bpath, header_lines)
    key = (name, layer, level)
    if key not in idx:
        raise HycError(-1, f"{name} layer {layer} level {level} not in {bpath}")
    rec, blo, bhi = idx[key]
    lo, hi = read_record(apath, rec, idm, jdm, nbdy, out)
    _check(lib().hyc_za_check(lo, hi, blo, bhi))
    return out


def write_record_file(path: str, fields, idm: int, jdm: int):
    """Write idm x jdm fields (numpy, (jdm, idm)) as a .a file: big-endian
    real*4 records padded to a multiple of 4096 words (test and tooling
    helper; HYCOM writes these with zaiowr)."""
    n2drec = (idm * jdm + 4095) // 4096 * 4096
    with open(path, "wb") as f:
        for a in fields:
            rec = np.zeros(n2drec, dtype=">f4")
            rec[:idm * jdm] = np.asarray(a, dtype=np.float64).reshape(-1).astype(">f4")
            f.write(rec.tobytes())
