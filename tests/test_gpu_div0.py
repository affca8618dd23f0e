"""The face kernels' zero-dividend division (gbf::div0 in gbf_physics.cuh)
returns the IEEE quotient bit for bit: run on the GPU beside the IEEE division
(libgbfprobe.so, gbf_probe_div0) over every pair of special operands (signed
zeros, subnormals, the largest and smallest normals, infinities, NaN) and
seeded random pairs, zero dividends included."""
import ctypes
import itertools

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def probe():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from jaxfluids_gb300 import build
    lib = ctypes.CDLL(build.build_probe())
    f = lib.gbf_probe_div0
    f.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_longlong, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


SPECIAL = [0.0, -0.0, 1.0, -1.0, 1.5, -2.75, 1e-30, 1e30, 5e-324, -5e-324, 2.2250738585072014e-308,
           -1e-310, 1.7976931348623157e308, -1.7976931348623157e308, float("inf"), float("-inf"), float("nan")]


def test_div0_equals_the_ieee_division_bitwise(probe):
    pairs = list(itertools.product(SPECIAL, SPECIAL))
    rng = np.random.default_rng(17)
    m = 200000
    ra = rng.standard_normal(m) * 10.0 ** rng.integers(-300, 300, m)
    rb = rng.standard_normal(m) * 10.0 ** rng.integers(-300, 300, m)
    ra[::3] = 0.0          # zero dividends over random divisors
    ra[1::7] = -0.0
    a = np.concatenate([np.array([p[0] for p in pairs]), ra])
    b = np.concatenate([np.array([p[1] for p in pairs]), rb])
    da = torch.from_numpy(a).cuda()
    db = torch.from_numpy(b).cuda()
    q0 = torch.empty_like(da)
    q1 = torch.empty_like(da)
    st = torch.cuda.current_stream().cuda_stream
    assert probe(da.data_ptr(), db.data_ptr(), q0.data_ptr(), q1.data_ptr(), a.size, st) == 0
    torch.cuda.synchronize()
    b0 = q0.cpu().numpy().view(np.uint64)
    b1 = q1.cpu().numpy().view(np.uint64)
    assert np.array_equal(b0, b1)
    # the zero-dividend cases are there, with both signs of zero in the results
    zq = q1.cpu().numpy()[(a == 0.0) & np.isfinite(b) & (b != 0.0)]
    assert zq.size > 50000 and np.all(zq == 0.0)
    assert np.any(np.signbit(zq)) and np.any(~np.signbit(zq))
