"""The position of a CD creation inside a strand, on the quantised rates.

The reference splits a strand of N1 Kuhn steps at newn = floor(0.5 + pr (N1 - 2)
/ w) + 1 (common/ensemble_kernel.cu:386).  The FP32 mirror of the oracle and the
sm_103a kernel evaluate it exactly on the quantised pick remainder r < w:
x = floor((2 r (N1 - 2) + w) / (2 w)).  The oracle uses 128-bit integers
(orc_split); the kernel (split_pos in dsm_kernels.cu) corrects an FP32 estimate
with 128-bit integer products.  Both are checked here against Python's
unbounded integers, the kernel's through a numpy restatement of its steps; the
device code itself is covered by the bit-exact GPU parity tests."""
import numpy as np


def exact(r: int, w: int, n1: int) -> int:
    m = max(n1 - 2, 0)
    if m == 0 or w == 0:
        return 0
    return (2 * r * m + w) // (2 * w)


def split_pos(r: int, w: int, n1: int) -> int:
    """The steps of split_pos: FP32 estimate, then exact correction."""
    m = max(n1 - 2, 0)
    if m == 0 or w == 0:
        return 0
    num = 2 * r * m + w
    d = 2 * w
    lz = 64 - w.bit_length()
    sh = max(0, 40 - lz)
    ratio = np.float32(np.float32(r >> sh) / np.float32(w >> sh))
    # the kernel's fma rounds once: ratio * m + 0.5 is exact in float64 (at most
    # 48 significant bits), so one rounding to float32 reproduces it
    q = int(np.float32(float(ratio) * float(np.float32(m)) + 0.5))
    q = min(max(q, 0), m)
    steps = 0
    while q * d > num:
        q -= 1
        steps += 1
    while (q + 1) * d <= num:
        q += 1
        steps += 1
    assert steps <= 2, (r, w, n1, steps)
    return q


def _cases():
    rng = np.random.default_rng(5)
    out = []
    for bits in (1, 8, 24, 25, 32, 40, 47, 48, 50):
        for _ in range(400):
            w = int(rng.integers(1, 1 << bits, dtype=np.uint64)) if bits < 64 else 1
            r = int(rng.integers(0, w, dtype=np.uint64)) if w > 1 else 0
            n1 = int(rng.integers(1, 6000))
            out.append((r, w, n1))
    # exact ties: 2 r m = (2k - 1) w
    for m in (1, 2, 3, 7, 100, 1999):
        for k in (1, 2, m):
            w = 2 * m * 1000003
            r = (2 * k - 1) * w // (2 * m)
            if r < w:
                out.append((r, w, m + 2))
                out.append((r - 1, w, m + 2))
                out.append((min(r + 1, w - 1), w, m + 2))
    out += [(0, 1, 2), (0, 5, 1), (4, 5, 3), ((1 << 48) - 2, (1 << 48) - 1, 5000), (0, 1 << 48, 200)]
    return out


def test_oracle_split_is_exact(oracle_mod):
    L = oracle_mod.lib()
    for r, w, n1 in _cases():
        assert L.orc_split(r, w, n1) == exact(r, w, n1), (r, w, n1)


def test_kernel_split_steps_are_exact():
    for r, w, n1 in _cases():
        assert split_pos(r, w, n1) == exact(r, w, n1), (r, w, n1)
