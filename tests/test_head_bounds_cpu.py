"""The error bound behind the tensor-core head phase (head_mma.cu), checked
on the CPU.

The head-score kernel multiplies TF32 operands (10 explicit mantissa bits)
and accumulates in FP32; the select kernel trusts that every score s~ lies
within (2^-9 + 2^-14) * |q||x| of the exact dot product, and that the
interval built from it holds the search kernel's exact distance.  Here the
worst case of the conversion -- every operand truncated toward zero -- and
accumulations that round toward zero after every 8-term block are simulated
in numpy, and the intervals (the kernel's formulas, in FP32) are checked to
contain the oracle's kernel distance, bit-exact arithmetic of the search.
CPU only."""
import numpy as np
import pytest

REL = np.float32(2.0 ** -9 + 2.0 ** -14)
SLACK = np.float32(2.0 ** -15)


def tf32_truncate(a):
    """Keep 10 mantissa bits, dropping the rest (rounding toward zero)."""
    b = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32) & np.uint32(0xFFFFE000)
    return b.view(np.float32)


def rz32(x):
    """float64 -> float32 rounded toward zero."""
    f = np.float32(x)
    return np.where(np.abs(f.astype(np.float64)) > np.abs(x), np.nextafter(f, np.float32(0)), f).astype(np.float32)


def worst_scores(q, x):
    """q . x with truncated operands and an accumulator rounded toward zero
    after every 8-term block (both pessimistic for a TF32 tensor core)."""
    qt, xt = tf32_truncate(q).astype(np.float64), tf32_truncate(x).astype(np.float64)
    acc = np.zeros((q.shape[0], x.shape[0]), np.float64)
    for k0 in range(0, q.shape[1], 8):
        blk = qt[:, k0:k0 + 8] @ xt[:, k0:k0 + 8].T
        acc = rz32(acc + blk).astype(np.float64)
    return acc.astype(np.float32)


def interval(metric, s, qn2, xn2):
    """The kernel's head_interval, in FP32 (head_mma.cu)."""
    f = np.float32
    qn, xn = np.sqrt(qn2).astype(f), np.sqrt(xn2).astype(f)
    e = (REL * qn * xn + f(1e-30)).astype(f)
    if metric == 0:
        d = (qn2 + xn2 - f(2) * s).astype(f)
        eps = (f(2) * e + SLACK * (qn2 + xn2 + f(2) * np.abs(s))).astype(f)
        return d - eps, d + eps
    if metric == 1:
        eps = (e + SLACK * qn * xn).astype(f)
        return -s - eps, -s + eps
    et = (e + SLACK * qn * xn).astype(f)
    tp, tm = (s + et).astype(f), (s - et).astype(f)
    with np.errstate(divide="ignore", invalid="ignore"):  # zero rows are handled below
        a = (-tp * np.abs(tp) / xn2).astype(f)
        b = (-tm * np.abs(tm) / xn2).astype(f)
    lo = a - SLACK * np.abs(a) - f(1e-30)
    hi = b + SLACK * np.abs(b) + f(1e-30)
    zero = ~(xn2 > f(1e-30))
    return np.where(zero, -np.inf, lo).astype(f), np.where(zero, np.inf, hi).astype(f)


def _data(kind, n, dim, seed):
    rng = np.random.default_rng(seed)
    if kind == "byte":
        c = rng.integers(0, 200, size=(8, dim))
        return np.clip(c[rng.integers(0, 8, n)] + rng.normal(0, 20, (n, dim)), 0, 255).round().astype(np.float32)
    if kind == "unit":
        v = rng.normal(0, 1, (n, dim)).astype(np.float32)
        return v / np.linalg.norm(v, axis=1, keepdims=True)
    # mantissas just below a TF32 boundary: every truncation loses almost 2^-10
    v = rng.uniform(1, 2, (n, dim)).astype(np.float32)
    b = v.view(np.uint32) | np.uint32(0x1FFF)
    return (b.view(np.float32) * rng.choice([-1, 1], (n, dim))).astype(np.float32)


@pytest.mark.parametrize("kind,dim", [("byte", 128), ("unit", 96), ("edge", 128), ("edge", 260), ("unit", 32)])
def test_truncated_scores_stay_within_the_bound(kind, dim):
    q, x = _data(kind, 64, dim, dim), _data(kind, 200, dim, dim + 1)
    s = worst_scores(q, x).astype(np.float64)
    exact = q.astype(np.float64) @ x.astype(np.float64).T
    scale = np.linalg.norm(q.astype(np.float64), axis=1)[:, None] * np.linalg.norm(x.astype(np.float64), axis=1)
    ratio = np.abs(s - exact) / np.maximum(scale, 1e-300)
    assert ratio.max() <= float(REL), ratio.max()


@pytest.mark.parametrize("metric", [0, 1, 2])
@pytest.mark.parametrize("kind,dim", [("byte", 128), ("unit", 96), ("edge", 64)])
def test_intervals_hold_the_kernel_distance(oracle, metric, kind, dim):
    q, x = _data(kind, 24, dim, 3 * dim + metric), _data(kind, 120, dim, 3 * dim + metric + 1)
    x[5] = 0.0  # a zero row: the cosine distance is 0 by the kernel's rule
    s = worst_scores(q, x)
    qn2 = np.einsum("ij,ij->i", q, q, dtype=np.float32)[:, None]
    xn2 = np.einsum("ij,ij->i", x, x, dtype=np.float32)[None, :]
    lo, hi = interval(metric, s, qn2.astype(np.float32), xn2.astype(np.float32))
    for i in range(q.shape[0]):
        for j in range(x.shape[0]):
            d = np.float32(oracle.kernel_distance(metric, q[i], x[j]))
            assert lo[i, j] <= d <= hi[i, j], (i, j, lo[i, j], d, hi[i, j])


def test_bf16_round_down_keeps_a_lower_bound():
    """The select kernel reads the lower bounds as BF16 rounded toward -inf
    (__float2bfloat16_rd), widened back exactly by a 16-bit shift: emulated
    here, every widened bound is <= the FP32 bound it came from and differs
    by less than one BF16 step."""
    rng = np.random.default_rng(4)
    v = np.concatenate([rng.normal(0, 1e6, 5000), rng.normal(0, 1, 5000), [0.0, -0.0, 1e-40, -1e-40]]).astype(np.float32)
    bits = v.view(np.uint32)
    trunc = bits & np.uint32(0xFFFF0000)  # toward zero
    neg_inexact = (v < 0) & (trunc != bits)
    down = np.where(neg_inexact, trunc + np.uint32(0x10000), trunc)  # one BF16 step further from zero
    widened = down.view(np.float32)  # the stored half in the high 16 bits, as the kernel widens it
    assert (widened <= v).all()
    step = np.abs(v.astype(np.float64)) * 2.0 ** -7 + 1e-38
    assert (v.astype(np.float64) - widened.astype(np.float64) <= step).all()
