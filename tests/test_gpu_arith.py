"""Device arithmetic that replaces a hardware operation must give its bits.

The final RK4 combination of the reference divides by 6
(JAX_BSSN/evolution/time_evolve.py:144-217).  The stage kernel forms that
quotient with one Markstein correction (three FP64 operations) instead of the
hardware division; the result has to equal the correctly rounded division bit
for bit on every input, since the state it updates is compared bitwise.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(n_random: int) -> np.ndarray:
    rng = np.random.default_rng(20261203)
    # log-uniform magnitudes over most of the double range, random signs
    mags = np.exp2(rng.uniform(-1000.0, 1000.0, n_random))
    random = mags * rng.choice([-1.0, 1.0], n_random)
    # the increments the RK4 step actually divides: dt * (k1 + 2k2 + 2k3 + k4)
    increments = rng.uniform(-1.0, 1.0, n_random) * np.exp2(rng.uniform(-60.0, 4.0, n_random))
    # raw bit patterns: every mantissa pattern in a few binades near one
    bits = (rng.integers(0, 1 << 52, n_random, dtype=np.int64)
            | (rng.integers(1020, 1030, n_random, dtype=np.int64) << 52)).view(np.float64)
    # exact multiples of 6 and their neighbours, integers, powers of two
    ints = np.arange(-100000, 100000, dtype=np.float64)
    sixes = 6.0 * rng.integers(1, 1 << 50, 100000).astype(np.float64)
    near = np.concatenate([np.nextafter(sixes, np.inf), np.nextafter(sixes, -np.inf)])
    pow2 = np.exp2(np.arange(-1074, 1024, dtype=np.float64))
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324, 2.2250738585072014e-308,
                        1.7976931348623157e308, -1.7976931348623157e308, 6.0, 1.0, 3.0, 12.0])
    return np.concatenate([random, increments, bits, ints, sixes, near, pow2, -pow2, special])


def test_division_by_six_matches_hardware(cuda, native):
    import torch
    from jax_bssn_gb300 import _native

    a_host = _inputs(1 << 21)
    a = torch.from_numpy(a_host).to(cuda)
    fast = torch.empty_like(a)
    hw = torch.empty_like(a)
    stream = torch.cuda.current_stream(cuda).cuda_stream
    _native.check(native.bssn_check_div6(a.data_ptr(), fast.data_ptr(), hw.data_ptr(), a.numel(), stream),
                  "bssn_check_div6")
    torch.cuda.synchronize(cuda)
    f = fast.cpu().numpy()
    h = hw.cpu().numpy()
    nan = np.isnan(h)
    assert np.array_equal(np.isnan(f), nan)
    mismatch = f[~nan].view(np.int64) != h[~nan].view(np.int64)
    assert not mismatch.any(), a_host[~nan][mismatch][:8]
    # and the hardware quotient is the correctly rounded one numpy gives
    assert np.array_equal(h[~nan].view(np.int64), (a_host[~nan] / 6.0).view(np.int64))
