"""The integer-instruction double <-> float conversions the mixed kernels use instead of
conversion instructions (df64.cuh: f32_of_f64, f64_of_f32, f2_split, f2_to_double) return the
hardware round-to-nearest results bit for bit: random bit patterns over every exponent, random
normal values, and the rounding and range edges (ties to even, carries into the exponent, the
float overflow and underflow thresholds, zeros, subnormals, inf, NaN)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _edges():
    f32max = float(np.finfo(np.float32).max)
    f32min = float(np.finfo(np.float32).tiny)
    vals = [0.0, -0.0, 1.0, -1.0, 0.1, 1.0 / 3.0, f32max, -f32max, f32min, -f32min,
            np.nextafter(f32min, 0.0), np.nextafter(f32min, 1.0), 2.0 ** -149, 2.0 ** -150,
            2.0 ** 127, 2.0 ** 128, np.inf, -np.inf, np.nan, 5e-324, 1.7976931348623157e308,
            2.0 ** -100, 2.0 ** -101, 2.0 ** 126, 2.0 ** 125 * 1.9999999]
    pats = []
    for e in (896, 897, 898, 1000, 1023, 1100, 1148, 1149, 1150, 1151):
        for m in (0, 1, 0x0FFFFFFF, 0x10000000, 0x10000001, 0x1FFFFFFF, 0x20000000, 0x30000000,
                  (1 << 52) - 1, (1 << 52) - 0x10000000, (1 << 52) - 0x20000000):
            for s in (0, 1):
                pats.append((s << 63) | (e << 52) | m)
    # the largest double below the float overflow threshold and the threshold itself
    pats.append(0x47EFFFFFEFFFFFFF)
    pats.append(0x47EFFFFFF0000000)
    return np.concatenate([np.array(vals, dtype=np.float64),
                           np.array(pats, dtype=np.uint64).view(np.float64)])


def test_integer_conversions_match_hardware(cuda):
    torch = cuda
    import gbmv
    rng = np.random.default_rng(11)
    raw = rng.integers(0, 2 ** 64 - 1, size=1 << 20, dtype=np.uint64, endpoint=True).view(np.float64)
    normal = rng.standard_normal(1 << 20) * 10.0 ** rng.uniform(-40, 40, size=1 << 20)
    for arr in (raw, normal, _edges()):
        d = torch.from_numpy(np.ascontiguousarray(arr)).cuda()
        assert gbmv.convert_check(d) == 0
