"""CPU checks of the C ABI: the library builds, loads, exports every entry
point the header declares, and its host-side logic (bigrid, argument and
mask validation) behaves without a GPU."""
import os
import re

import numpy as np
import pytest

import hycadv
from helpers import basin, oracle_grid

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "hycom_adv.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(hyc_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(built_lib):
    L = hycadv.lib()
    declared = header_functions()
    assert declared, "no declarations found"
    for name in declared:
        assert hasattr(L, name), f"{name} declared in include/hycom_adv.h but not exported"
    assert set(declared) == set(hycadv.EXPORTS)
    assert "sm_103a" in hycadv.version()


@pytest.mark.parametrize("periodic,nx,ny,seed", [(False, 61, 47, 3), (True, 64, 40, 5), (False, 257, 193, 7)])
def test_bigrid_matches_oracle(built_lib, periodic, nx, ny, seed):
    b = basin(nx, ny, periodic, seed)
    g = oracle_grid(b)
    depth_after, masks, nreg = hycadv.bigrid(b.depth, b.nbdy)
    assert nreg == g.nreg
    for k in ("ip", "iu", "iv", "ipim1", "ipip1", "ipjm1", "ipjp1"):
        assert np.array_equal(masks[k], g.masks[k]), k
    assert np.array_equal(depth_after, g.depth)


def test_bigrid_rejects_one_point_sea(built_lib):
    b = basin(30, 20, False, seed=1)
    d = b.depth.copy()
    d[b.J, b.I] = 0.0
    d[b.nbdy + 10, b.nbdy + 10] = 100.0  # isolated sea cell
    with pytest.raises(hycadv.HycError) as e:
        hycadv.bigrid(d, b.nbdy)
    assert e.value.code == -7


def test_init_rejects_inconsistent_masks(built_lib):
    b = basin(30, 20, False, seed=2)
    _, m, nreg = hycadv.bigrid(b.depth, b.nbdy)
    iu = m["iu"].copy()
    iu[b.nbdy + 5, b.nbdy + 5] ^= 1
    sc, si = b.metrics()
    with pytest.raises(hycadv.HycError) as e:
        hycadv.Context(b.nx, b.ny, 2, b.nbdy, nreg, m["ip"], iu, m["iv"], sc, si)
    assert e.value.code == -4
    assert "iu(" in str(e.value)


def test_init_argument_errors(built_lib):
    b = basin(30, 20, False, seed=2)
    _, m, nreg = hycadv.bigrid(b.depth, b.nbdy)
    sc, si = b.metrics()
    with pytest.raises(hycadv.HycError) as e:
        hycadv.Context(b.nx, b.ny, 2, 2, nreg, m["ip"], m["iu"], m["iv"], sc, si)  # nbdy < 3
    assert e.value.code == -1
    with pytest.raises(hycadv.HycError) as e:
        hycadv.Context(b.nx, b.ny, 2, b.nbdy, 2, m["ip"], m["iu"], m["iv"], sc, si)  # nreg 2 (arctic)
    assert e.value.code == -1


def test_init_without_gpu_fails_loudly(built_lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    b = basin(30, 20, False, seed=2)
    _, m, nreg = hycadv.bigrid(b.depth, b.nbdy)
    sc, si = b.metrics()
    with pytest.raises(hycadv.HycError) as e:
        hycadv.Context(b.nx, b.ny, 2, b.nbdy, nreg, m["ip"], m["iu"], m["iv"], sc, si)
    assert e.value.code == -5
