"""The C-ABI library builds, loads and exports every declared symbol; host-side
argument handling mirrors the reference.  No GPU needed."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    out = []
    for f in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            out += re.findall(r"\b(pyl_\w+)\s*\(", src)
    return sorted(set(out))


@pytest.fixture(scope="module")
def lib():
    from pylians3_gb300 import build_native, _native
    build_native.build()
    return _native.load()


def test_every_declared_symbol_is_exported(lib):
    from pylians3_gb300 import _native
    syms = declared_symbols()
    assert len(syms) >= 15
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    assert sorted(set(_native.EXPORTS) | set(syms)) == sorted(set(_native.EXPORTS)), \
        "binding table out of date"


@pytest.mark.parametrize("dims", [2, 3, 16, 17, 64, 128, 192, 256, 384, 512, 1024])
def test_pk_sizes_match_frequencies(lib, dims):
    from pylians3_gb300 import _native, Pk_library as PKL
    kmax, kmax_par, kmax_per = _native.pk_sizes(dims)
    _, _, kp, kq, km = PKL.frequencies(1000.0, dims)
    assert (kmax, kmax_par, kmax_per) == (km, kp, kq)


def test_reference_helpers():
    from pylians3_gb300 import Pk_library as PKL
    from oracle import oracle as orc
    for m in ("NGP", "CIC", "TSC", "PCS", "None", "xyz"):
        assert PKL.MAS_function(m) == orc.MAS_function(m)
    assert PKL.MAS_correction(0.0, 2) == 1.0
    x = 0.3
    assert PKL.MAS_correction(x, 3) == pytest.approx((x / np.sin(x)) ** 3, rel=1e-15)
    assert PKL.frequencies(1000.0, 128) == orc.frequencies(1000.0, 128)
    with pytest.raises(SystemExit):
        PKL.check_number_modes(np.ones(5), 8)


def test_ma_argument_errors_behave_like_reference(lib, capsys):
    from pylians3_gb300 import MAS_library as MASL
    pos = np.zeros((10, 3), np.float32)
    with pytest.raises(SystemExit):
        MASL.MA(pos, np.zeros((8, 8), np.float32), 1.0, "CIC")
    assert "pos have 3 dimensions and the density 2" in capsys.readouterr().out
    with pytest.raises(SystemExit):
        MASL.MA(pos, np.zeros((8, 8, 8), np.float32), 1.0, "XYZ")
    assert "option not valid" in capsys.readouterr().out
    with pytest.raises(ValueError):
        MASL.MA(pos.astype(np.float64), np.zeros((8, 8, 8), np.float32), 1.0, "CIC")
    with pytest.raises(ValueError):
        MASL.CIC(pos, np.zeros((8, 8, 8), np.float64), 1.0)


def test_pk_argument_errors(lib):
    from pylians3_gb300 import Pk_library as PKL
    with pytest.raises(ValueError):
        PKL.Pk(np.zeros((8, 8, 8), np.float64), 1.0, verbose=False)
    with pytest.raises(ValueError):
        PKL.Pk(np.zeros((8, 8, 4), np.float32), 1.0, verbose=False)


def test_no_gpu_reports_cuda_error(lib):
    """Without a device the context creation fails with a status, not a crash."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    p = ctypes.c_void_p()
    rc = lib.pyl_ctx_create(ctypes.byref(p), 0, None)
    assert rc != 0 and not p.value


def test_product_never_imports_the_oracle():
    pkg = os.path.join(ROOT, "pylians3_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h")):
                src = open(os.path.join(dirpath, f)).read()
                assert "import oracle" not in src and "from oracle" not in src, f
                assert "liborc" not in src, f


def test_tile_shape_validation():
    """pyl_set_tile_shape checks shapes on the host (no GPU needed)."""
    import ctypes
    from pylians3_gb300 import _native as N
    lib = N.load()
    v = [ctypes.c_int() for _ in range(4)]
    assert lib.pyl_get_tile_shape(512, 2, *[ctypes.byref(x) for x in v]) == N.PYL_OK
    default = [x.value for x in v]
    assert lib.pyl_set_tile_shape(512, 2, 12, 32, 32, 0) == N.PYL_ERR_ARG       # not 2^k
    assert lib.pyl_set_tile_shape(512, 4, 64, 64, 64, 0) == N.PYL_ERR_UNSUPPORTED  # footprint
    assert lib.pyl_set_tile_shape(512, 2, 8, 8, 16, 0) == N.PYL_ERR_UNSUPPORTED   # > 256 buckets
    assert lib.pyl_set_tile_shape(512, 2, 32, 32, 32, 16) == N.PYL_OK
    lib.pyl_get_tile_shape(512, 2, *[ctypes.byref(x) for x in v])
    assert [x.value for x in v] == [32, 32, 32, 16]
    assert lib.pyl_set_tile_shape(512, 2, 0, 0, 0, 0) == N.PYL_OK
    lib.pyl_get_tile_shape(512, 2, *[ctypes.byref(x) for x in v])
    assert [x.value for x in v] == default
