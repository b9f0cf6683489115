"""HYCOM .a/.b input (zaiord, restart_in3d): big-endian real*4 records
padded to 4096 words, masked and unmasked reads, the 2^100 data void, the
.b range check.  CPU only."""
import numpy as np
import pytest

import hycadv
from hycadv import za

SPVAL = np.float32(2.0 ** 100)


def fields(idm, jdm, n, seed=5):
    rng = np.random.default_rng(seed)
    return [rng.normal(10.0 * (k + 1), 3.0, (jdm, idm)).astype(np.float32).astype(np.float64) for k in range(n)]


def test_records_round_trip(tmp_path, built_lib):
    idm, jdm, nb = 70, 50, 3  # 3500 words: records padded to 4096
    fs = fields(idm, jdm, 3)
    fs[1][7, 9] = SPVAL  # a data void
    a = str(tmp_path / "f.a")
    za.write_record_file(a, fs, idm, jdm)
    assert (tmp_path / "f.a").stat().st_size == 3 * 4096 * 4
    for r, f in enumerate(fs, start=1):
        out = np.full((jdm + 2 * nb, idm + 2 * nb), -7.0)
        lo, hi = za.read_record(a, r, idm, jdm, nb, out)
        assert np.array_equal(out[nb:-nb, nb:-nb], f)
        assert np.all(out[:nb] == -7.0) and np.all(out[:, :nb] == -7.0)  # halo untouched
        good = f[f != SPVAL]
        assert lo == good.min() and hi == good.max()


def test_masked_read(tmp_path, built_lib):
    idm, jdm, nb = 40, 30, 2
    f = fields(idm, jdm, 1)[0]
    mask = np.zeros((jdm + 2 * nb, idm + 2 * nb), np.int32)
    mask[nb + 3:nb + 20, nb + 5:nb + 30] = 1
    f[0, 0] = SPVAL  # void outside the mask: allowed
    a = str(tmp_path / "m.a")
    za.write_record_file(a, [f], idm, jdm)
    out = np.zeros_like(mask, dtype=np.float64)
    lo, hi = za.read_record(a, 1, idm, jdm, nb, out, mask=mask)
    inside = mask[nb:-nb, nb:-nb] != 0
    assert np.array_equal(out[nb:-nb, nb:-nb][inside], f[inside])
    assert np.all(out[nb:-nb, nb:-nb][~inside] == 0.0)
    assert lo == f[inside].min() and hi == f[inside].max()
    f[5, 10] = SPVAL  # void inside the mask: zaiord stops
    za.write_record_file(a, [f], idm, jdm)
    with pytest.raises(hycadv.HycError):
        za.read_record(a, 1, idm, jdm, nb, out, mask=mask)


def test_restart_pair_and_range_check(tmp_path, built_lib):
    idm, jdm, nb = 33, 21, 2
    fs = fields(idm, jdm, 4, seed=9)
    names = [("temp", 1, 1), ("temp", 2, 1), ("saln", 1, 1), ("saln", 2, 1)]
    a, b = str(tmp_path / "restart_in.a"), str(tmp_path / "restart_in.b")
    za.write_record_file(a, fs, idm, jdm)
    with open(b, "w") as fb:
        fb.write("RESTART2: iexpt,iversn,yrflag,sigver =    10    22     3     2\n")
        fb.write("RESTART2: nstep,dtime,thbase = 100 1.0 34.0\n")
        for (nm, lay, lev), f in zip(names, fs):
            fb.write(f"{nm:<8s}: layer,tlevel,range = {lay:3d} {lev:2d} {f.min(): .6E} {f.max(): .6E}\n")
    out = np.zeros((jdm + 2 * nb, idm + 2 * nb))
    za.read_restart_field(a, b, "saln", 2, 1, idm, jdm, nb, out)
    assert np.array_equal(out[nb:-nb, nb:-nb], fs[3])
    assert za.parse_b("temp    : layer,tlevel,range =   3  2  -1.5E+00  2.5E+01")[:3] == ("temp    ", 3, 2)
    # a .b range that disagrees with the data is an error (mod_restart.F90:604-605)
    with open(b) as fb:
        lines = fb.read().splitlines()
    lines[2 + 1] = lines[2 + 1].rsplit(" ", 1)[0] + " 9.9E+09"
    with open(b, "w") as fb:
        fb.write("\n".join(lines) + "\n")
    with pytest.raises(hycadv.HycError):
        za.read_restart_field(a, b, "temp", 2, 1, idm, jdm, nb, out)
    with pytest.raises(hycadv.HycError):
        za.read_record(a, 5, idm, jdm, nb, out)  # past the end
