"""The digit split of the tensor-core FP64-accurate product, on the host
(ipt_block_accurate_split_host, the same code the kernels run) against the
oracle's restatement: exponents and digits bit for bit, the digits
reconstruct the rounded fixed-point value, and the rounding error is at
most half a unit of 2^(e - 48)."""
import ctypes as C

import numpy as np

from oracle import oracle


def host_split(lib, v, max_abs):
    v = np.ascontiguousarray(v, dtype=np.float64)
    e = C.c_int(0)
    out = np.zeros((v.size, 6), dtype=np.int32)
    st = lib.ipt_block_accurate_split_host(C.c_void_p(v.ctypes.data), v.size, float(max_abs),
                                          C.byref(e), C.c_void_p(out.ctypes.data))
    assert st == 0
    return e.value, out


def cases():
    rng = np.random.default_rng(1)
    yield rng.standard_normal(257) * 0.02
    yield rng.standard_normal(100) * np.exp(-rng.uniform(0, 60, 100))  # wide dynamic range
    yield np.array([1.0, -1.0, 0.5, 0.75, -0.999999, 2.0 ** -60, 0.0, -0.0])
    yield np.array([3.0, -2.9999999999, 1.5, 2.0 ** -40])
    yield np.array([5e-324, 1e-310, -2.2e-308, 0.0])  # subnormal rows
    yield rng.uniform(-1, 1, 64) * 1e300
    x = rng.standard_normal(50)
    x[7] = 0.5 * 2.0 ** -48 * 4  # ties and exact powers
    yield x


def test_split_matches_oracle(lib):
    for v in cases():
        mx = np.abs(v).max()
        e, d = host_split(lib, v, mx)
        assert e == oracle.accurate_exponent(mx)
        q = oracle.accurate_fixed(v, e)
        np.testing.assert_array_equal(d, oracle.accurate_digits(q))
        # digit ranges and reconstruction
        assert np.abs(d[:, 0]).max() <= 256 and (d[:, 1:] >= -128).all() and (d[:, 1:] <= 127).all()
        rec = [sum(int(d[i, s]) << (8 * (5 - s)) for s in range(6)) for i in range(len(v))]
        assert rec == q.tolist()
        # round to nearest at the scale 2^(e - 48)
        for vi, qi in zip(v.tolist(), rec):
            exact = np.ldexp(vi, 48 - e) if vi != 0 else 0.0
            assert abs(exact - qi) <= 0.5 + 1e-9


def test_split_nonfinite_row(lib):
    e, d = host_split(lib, np.array([1.0, np.nan, np.inf]), np.inf)
    assert e == 0x7FFFFFFF and not d.any()


def test_fast_digit_extraction_is_identical(tmp_path):
    """The kernels' 32-bit digit extraction (oz_digits_fast) equals the 64-bit
    definition (oz_digits_of of oz_fixed) on 3 million values (compiled with
    the host C++ compiler from the library's own header)."""
    import os
    import shutil
    import subprocess
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        import pytest
        pytest.skip("no C++ compiler")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = str(tmp_path / "oz_eq")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", os.path.join(root, "block_ipt_gb300", "csrc"),
                    os.path.join(root, "tests", "cpp", "oz_digits_equivalence.cpp"), "-o", exe],
                   check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    assert "mismatches 0" in out.stdout
