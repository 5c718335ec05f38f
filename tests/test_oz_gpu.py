"""The FP64-accurate products of the mixed refinement, r = b - A x and
g = A^T r (rnpgpu_dls_residual), formed on the tensor cores from exact
fixed-point slices: against extended-precision references (numpy longdouble,
at least 64-bit significands) with the error bound of the slicing,
2^-53 of sum_k 2^e_k |x_kj| (e_k the power-of-two scale of column k), given
16x slack; exactness of the integer accumulation at its largest digit sums;
column scales across the whole exponent range; ragged sizes; several groups of
right-hand sides; NaN propagation."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from rnp2_gb300 import ls as gls  # noqa: E402

LD = np.longdouble


def to_dev(a):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64).T)).cuda().t()


def from_dev(t):
    return t.t().cpu().numpy().T


def col_scale(A):
    """2^e_k with |a_ik| < 2^(e_k - 1): the slicing's column scales."""
    mx = np.abs(A).max(axis=0)
    e = np.where(mx > 0, np.floor(np.log2(np.where(mx > 0, mx, 1.0))) + 2, -np.inf)
    return np.exp2(e)


def residual_bound(A, X):
    # 2^-49 * sum_k 2^e_k |x_kj|: the slicing's 2^-53 with 16x slack
    return np.exp2(-49) * (col_scale(A)[None, :] @ np.abs(X))


def run(A, X, B, normal=False):
    out = gls.residual(to_dev(A), to_dev(X), to_dev(B), normal=normal)
    torch.cuda.synchronize()
    if normal:
        return from_dev(out[0]), from_dev(out[1])
    return from_dev(out)


def exact_residual(A, X, B):
    return B.astype(LD) - A.astype(LD) @ X.astype(LD)


@pytest.mark.parametrize("mnr", [(1000, 300, 5), (128, 16, 16), (4096, 512, 16), (777, 700, 17), (1, 1, 1), (300, 1, 3), (2000, 33, 2)])
def test_residual_against_extended_precision(mnr):
    m, n, nrhs = mnr
    rng = np.random.default_rng(m * 7 + n)
    A = rng.standard_normal((m, n))
    X = rng.standard_normal((n, nrhs))
    B = A @ X + 1e-6 * rng.standard_normal((m, nrhs))
    R = run(A, X, B)
    err = np.abs(R.astype(LD) - exact_residual(A, X, B)).astype(np.float64)
    bound = np.broadcast_to(residual_bound(A, X), err.shape)
    assert np.all(err <= bound), float((err / bound).max())
    # and as accurate as an FP64 matrix product (within a small factor)
    err64 = np.abs((B - A @ X).astype(LD) - exact_residual(A, X, B)).astype(np.float64)
    assert err.max() <= 4 * err64.max() + np.exp2(-52) * np.abs(B).max()


def test_residual_normal_products():
    m, n, nrhs = 3000, 260, 7
    rng = np.random.default_rng(11)
    A = rng.standard_normal((m, n)) * np.exp2(rng.integers(-20, 20, size=n))[None, :]
    X = rng.standard_normal((n, nrhs))
    B = A @ X + 1e-3 * rng.standard_normal((m, nrhs))
    R, G = run(A, X, B, normal=True)
    err = np.abs(R.astype(LD) - exact_residual(A, X, B)).astype(np.float64)
    assert np.all(err <= residual_bound(A, X))
    # g = A^T r of the returned r: error below 2^-49 * m * 2^e_k * 2^f_j
    Gx = (A.astype(LD).T @ R.astype(LD)).astype(np.float64)
    rs = np.exp2(np.floor(np.log2(np.abs(R).max(axis=0))) + 2)
    bound = np.exp2(-49) * m * col_scale(A)[:, None] * rs[None, :]
    assert np.all(np.abs(G - Gx) <= bound)
    assert np.abs(G - Gx).max() <= 1e-9 * np.abs(Gx).max()


def test_largest_digit_sums_are_exact():
    # a = 126/127 has seven top digits 63 (the largest balanced digit); with
    # x the same and n = 512 every level of the accumulation reaches its
    # largest sum (level 7: 8 * 63^2 * 512 < 2^24), so any rounding in the
    # integer accumulation would show
    m, n, nrhs = 256, 512, 16
    A = np.full((m, n), 126.0 / 127.0)
    X = np.full((n, nrhs), 126.0 / 127.0)
    B = np.zeros((m, nrhs))
    R = run(A, X, B)
    ex = exact_residual(A, X, B)
    rel = np.abs((R.astype(LD) - ex) / ex).astype(np.float64)
    assert rel.max() <= 2.0 ** -50


def test_column_scales_span_the_exponent_range():
    m, n, nrhs = 700, 90, 4
    rng = np.random.default_rng(5)
    s = np.exp2(np.linspace(-900, 900, n).round())
    A = rng.standard_normal((m, n)) * s[None, :]
    X = rng.standard_normal((n, nrhs)) / s[:, None]
    B = rng.standard_normal((m, nrhs))
    R = run(A, X, B)
    err = np.abs(R.astype(LD) - exact_residual(A, X, B)).astype(np.float64)
    assert np.all(err <= residual_bound(A, X))


def test_zero_columns_and_right_hand_sides():
    m, n, nrhs = 500, 40, 3
    rng = np.random.default_rng(2)
    A = rng.standard_normal((m, n))
    A[:, 7] = 0.0
    A[:, 39] = 0.0
    X = rng.standard_normal((n, nrhs))
    X[:, 1] = 0.0
    B = rng.standard_normal((m, nrhs))
    R = run(A, X, B)
    assert np.array_equal(R[:, 1], B[:, 1])
    err = np.abs(R.astype(LD) - exact_residual(A, X, B)).astype(np.float64)
    assert np.all(err <= residual_bound(A, X))


def test_tiny_and_subnormal_entries():
    m, n, nrhs = 300, 20, 2
    rng = np.random.default_rng(3)
    A = rng.standard_normal((m, n)) * 1e-300
    A[5, 3] = 4e-320
    X = rng.standard_normal((n, nrhs)) * 1e290
    B = rng.standard_normal((m, nrhs)) * 1e-10
    R = run(A, X, B)
    err = np.abs(R.astype(LD) - exact_residual(A, X, B)).astype(np.float64)
    assert np.all(err <= residual_bound(A, X))


def test_nan_in_a_propagates():
    m, n, nrhs = 200, 30, 2
    rng = np.random.default_rng(4)
    A = rng.standard_normal((m, n))
    A[17, 4] = np.nan
    X = rng.standard_normal((n, nrhs))
    R = run(A, X, rng.standard_normal((m, nrhs)))
    assert np.isnan(R).all()


def test_nan_in_x_propagates_to_its_column():
    m, n, nrhs = 200, 30, 3
    rng = np.random.default_rng(6)
    A = rng.standard_normal((m, n))
    X = rng.standard_normal((n, nrhs))
    X[2, 1] = np.inf
    B = rng.standard_normal((m, nrhs))
    R = run(A, X, B)
    assert np.isnan(R[:, 1]).all()
    err = np.abs(R[:, [0, 2]].astype(LD) - exact_residual(A, X, B)[:, [0, 2]]).astype(np.float64)
    assert np.all(err <= residual_bound(A, X)[:, [0, 2]])


def test_in_place_and_repeatable():
    m, n, nrhs = 1500, 128, 16
    rng = np.random.default_rng(8)
    A = rng.standard_normal((m, n))
    X = rng.standard_normal((n, nrhs))
    B = rng.standard_normal((m, nrhs))
    dA, dX, dB = to_dev(A), to_dev(X), to_dev(B)
    R1 = gls.residual(dA, dX, dB)
    R2 = gls.residual(dA, dX, dB)
    gls.residual(dA, dX, dB, R=dB)  # r = b - A x written over b
    torch.cuda.synchronize()
    assert torch.equal(R1, R2)
    assert torch.equal(R1, dB)
