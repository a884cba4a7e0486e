"""The integer-pipe double -> (hi, lo) float split against numpy's IEEE
conversions: hi = float32(a), lo = float32(a - hi), bit for bit, on the host
restatement (CPU) and on the device kernel (GPU)."""
import ctypes as C

import numpy as np
import pytest

from block_ipt_gb300 import _lib


def edge_values():
    rng = np.random.default_rng(5)
    parts = [
        rng.standard_normal(20000) * 10.0 ** rng.uniform(-30, 30, 20000),
        rng.uniform(-1, 1, 5000) * 2.0 ** rng.integers(-160, -100, 5000),   # float subnormal range
        rng.uniform(-1, 1, 2000) * 2.0 ** rng.integers(-1074, -1000, 2000),  # double subnormal
        rng.uniform(-1, 1, 2000) * 2.0 ** rng.integers(100, 140, 2000),      # near float overflow
        np.array([0.0, -0.0, np.inf, -np.inf, 3.4028234663852886e38, 3.4028235677973366e38,
                  -3.4028235677973366e38, 1.1754943508222875e-38, 1.1754942106924411e-38,
                  2.0 ** -149, 2.0 ** -150, 2.0 ** -150 * 1.0000001, 1.0, -1.0, 2.0 ** -74,
                  2.0 ** -75, 1e-30, 1e30]),
    ]
    # exact ties of the 29 dropped mantissa bits, even and odd kept mantissas
    m = rng.integers(0, 2 ** 23, 4000, dtype=np.uint64)
    e = rng.integers(1023 - 126, 1023 + 127, 4000, dtype=np.uint64)
    bits = (e << np.uint64(52)) | (m << np.uint64(29)) | np.uint64(1 << 28)
    bits |= rng.integers(0, 2, 4000, dtype=np.uint64) << np.uint64(63)
    parts.append(bits.view(np.float64))
    # remainders that round inside lo (more than 24 significant bits left)
    bits = (e << np.uint64(52)) | rng.integers(0, 2 ** 52, 4000, dtype=np.uint64)
    parts.append(bits.view(np.float64))
    return np.concatenate(parts)


def numpy_split(a):
    with np.errstate(over="ignore", invalid="ignore"):
        hi = a.astype(np.float32)
        lo = (a - hi.astype(np.float64)).astype(np.float32)
    return hi, lo


def same_bits(x, y):
    nan = np.isnan(x) & np.isnan(y)
    return np.all((x.view(np.uint32) == y.view(np.uint32)) | nan)


def test_split_host_matches_ieee():
    a = edge_values()
    hi = np.empty(a.size, np.float32)
    lo = np.empty(a.size, np.float32)
    st = _lib.load().ipt_block_split_double_host(a.ctypes.data, a.size, hi.ctypes.data,
                                                 lo.ctypes.data)
    assert st == 0
    rh, rl = numpy_split(a)
    assert same_bits(hi, rh)
    assert same_bits(lo, rl)


def test_split_host_invalid():
    assert _lib.load().ipt_block_split_double_host(None, 4, None, None) != 0
    assert _lib.load().ipt_block_split_double_host(None, 0, None, None) == 0


@pytest.mark.gpu
def test_split_device_matches_ieee(cuda):
    torch = cuda
    a = edge_values()
    da = torch.from_numpy(a).cuda()
    hi = torch.empty(a.size, dtype=torch.float32, device="cuda")
    lo = torch.empty(a.size, dtype=torch.float32, device="cuda")
    st = _lib.load().ipt_block_split_double(C.c_void_p(da.data_ptr()), a.size,
                                            C.c_void_p(hi.data_ptr()), C.c_void_p(lo.data_ptr()),
                                            C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    torch.cuda.synchronize()
    rh, rl = numpy_split(a)
    assert same_bits(hi.cpu().numpy(), rh)
    assert same_bits(lo.cpu().numpy(), rl)

