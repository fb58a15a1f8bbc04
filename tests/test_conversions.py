"""The kernel's float -> 64-bit integer conversion built from 32-bit operations.

dsm_kernels.cu quantises the rate components that update_pairs recomputes
after each event with f2u64_rn instead of the 64-bit conversion instruction.
These tests replay its operations with numpy's IEEE single-precision
arithmetic and check them against exact round-to-nearest-even (llrint): every
float of [2^21, 2^24) (all ties and the carry into 2^24) and sampled floats of
every binade up to 2^63.  The device code itself is checked by the bit-exact
GPU parity tests, which depend on every conversion."""
import numpy as np

F32_2P23 = np.float32(8388608.0)


def f2u64_rn(y):
    """The operations of f2u64_rn on float32 inputs in [0, 2^63)."""
    b = y.view(np.uint32) & np.uint32(0x7FFFFFFF)
    e = (b >> np.uint32(23)).astype(np.int64) - 150
    small = ((b.view(np.float32) + F32_2P23).view(np.uint32) - np.uint32(0x4B000000)).astype(np.uint64)
    sig = ((b & np.uint32(0x7FFFFF)) | np.uint32(0x800000)).astype(np.uint64)
    big = sig << (e & 63).astype(np.uint64)
    return np.where(e < 0, small, big)


def test_f2u64_dense_ties():
    """Every float in [2^21, 2^24): halves, quarters, the carry at 2^23 - 0.5."""
    b = np.arange(0x4A000000, 0x4B800000, dtype=np.uint32)
    y = b.view(np.float32)
    got = f2u64_rn(y)
    want = np.rint(y.astype(np.float64)).astype(np.uint64)
    assert np.array_equal(got, want)


def test_f2u64_all_binades():
    """Random floats of every binade from the subnormals to 2^63, zero and -0.0."""
    rng = np.random.default_rng(11)
    b = rng.integers(0, 0x5F000000, size=4_000_000, dtype=np.uint32)
    b = np.concatenate([b, np.array([0, 1, 0x7FFFFF, 0x800000, 0x3F000000, 0x3FC00000, 0x5EFFFFFF], np.uint32)])
    y = b.view(np.float32)
    assert np.array_equal(f2u64_rn(y), np.rint(y.astype(np.float64)).astype(np.uint64))
    assert f2u64_rn(np.array([-0.0], np.float32))[0] == 0
