"""tcgen05 / FP32 Gram and cross products against FP64 NumPy."""
import numpy as np
import pytest

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

# rel-L2 vs FP64: FP32 SIMT and split tensor-core products 1e-5, one BF16 pass 1e-2
TOL = {"fp32": 1e-5, "split": 1e-5, "bf16": 1e-2}


@pytest.fixture(scope="module")
def ctx(gpu):
    from sid_gb300.nnls import Context
    return Context()


@pytest.mark.parametrize("P,K", [(5000, 300), (4097, 129), (640, 64), (70000, 800)])
@pytest.mark.parametrize("prec", ["fp32", "split", "bf16"])
def test_gram(ctx, P, K, prec):
    from sid_gb300 import to_numpy
    rng = np.random.default_rng(P + K)
    A = np.asfortranarray(rng.random((P, K), dtype=np.float32) * (rng.random(K) < 0.9))
    G = to_numpy(ctx.gram(A, prec))
    ref = A.astype(np.float64).T @ A.astype(np.float64)
    ctx.sync()
    assert rel_l2(G, ref) < TOL[prec], rel_l2(G, ref)


@pytest.mark.parametrize("P,K,F", [(7000, 200, 500), (3001, 77, 129), (100000, 800, 300)])
@pytest.mark.parametrize("prec", ["fp32", "split", "bf16"])
def test_cross_f32(ctx, P, K, F, prec):
    from sid_gb300 import to_numpy
    rng = np.random.default_rng(P * 7 + F)
    A = np.asfortranarray(rng.random((P, K), dtype=np.float32))
    Y = np.asfortranarray(rng.standard_normal((P, F)).astype(np.float32))
    h = to_numpy(ctx.cross(A, Y, prec))
    ref = A.astype(np.float64).T @ Y.astype(np.float64)
    ctx.sync()
    assert rel_l2(h, ref) < TOL[prec] * 10, rel_l2(h, ref)  # signed Y: cancellation


@pytest.mark.parametrize("P,K,F", [(7000, 200, 500), (3003, 77, 129)])
@pytest.mark.parametrize("prec", ["split", "bf16"])
def test_cross_f16_movie(ctx, P, K, F, prec):
    from sid_gb300 import to_numpy
    rng = np.random.default_rng(P + 3 * F)
    A = np.asfortranarray(rng.random((P, K), dtype=np.float32) * 0.01)
    Y = np.asfortranarray((rng.random((P, F)) * 100).astype(np.float16))
    h = to_numpy(ctx.cross(A, Y, prec))
    ref = A.astype(np.float64).T @ Y.astype(np.float64)
    ctx.sync()
    tol = {"split": 1e-5, "bf16": 2e-3}[prec]
    assert rel_l2(h, ref) < tol, rel_l2(h, ref)
