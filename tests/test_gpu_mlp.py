"""The learned preconditioner on the GPU: the tcgen05/TMA BF16 GEMM against
numpy, the network's forward/backward against the CPU oracle, and the
trained network inside flexible PCG against plain block-Jacobi PCG."""
import numpy as np
import pytest

import sanepic_gb300 as sg
from oracle import mlp
from sanepic_gb300 import build, synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    build.build()


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 256, 768), (384, 768, 256),
                                   (256, 256, 4096), (128, 512, 192)])
def test_gemm_matches_numpy(M, N, K):
    rng = np.random.default_rng(M + N + K)
    A = mlp.bf16_bits(rng.normal(size=(M, K)).astype(np.float32))
    B = mlp.bf16_bits(rng.normal(size=(N, K)).astype(np.float32))
    C, _ = sg.gemm_bf16(A, B)
    Af = (A.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    Bf = (B.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    ref = Af @ Bf.T
    # FP32 accumulation of K products of O(1) values
    tol = 1e-6 * np.sqrt(K) * np.abs(Af).max() * np.abs(Bf).max() * 8
    assert np.abs(C - ref).max() <= tol


def test_network_gradients_match_oracle():
    rng = np.random.default_rng(11)
    p = mlp.init_params(5, out_scale=0.5)
    X = rng.normal(size=(256, 768)).astype(np.float32)
    T = (rng.normal(size=(256, 768)) * 0.3).astype(np.float32)
    Y, loss, g = sg.mlp_grad(p, X, T)
    Yo, loss_o, go = mlp.forward_backward(p, X, T)
    # both sides follow the same BF16 rounding contract; what remains is the
    # FP32 accumulation order (measured: Y 1.4e-4, gradients 3e-5 .. 5e-4)
    assert np.linalg.norm(Y - Yo) / np.linalg.norm(Yo) < 1e-3
    assert abs(loss - loss_o) / loss_o < 1e-3
    offs = np.cumsum([0] + [o * i + o for i, o in zip(mlp.LAYER_IN, mlp.LAYER_OUT)])
    for l in range(4):
        a, b = g[offs[l]:offs[l + 1]], go[offs[l]:offs[l + 1]]
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < 2e-3, l
        assert np.dot(a, b) / (np.linalg.norm(a) * np.linalg.norm(b)) > 0.99999, l


def _rel(a, b, npix):
    """relative difference of two [I|Q|U] maps, the I monopole (a near-null mode
    of A with 1/f noise) removed"""
    d = a - b
    d[:npix] -= d[:npix].mean()
    return np.linalg.norm(d) / np.linalg.norm(b)


def test_learned_preconditioner_end_to_end():
    spec = synth.ProblemSpec("learn", ndet=8, nside=32, nseg=8, ns=8192, fknee=0.1, alpha=1.5,
                             problem=21, precision="f32")
    prob = synth.make_problem(spec)
    mm = sg.from_problem(prob, precision="f32")
    npix = mm.npix
    # trained and judged by plain PCG on a held-out problem
    rep = mm.learn_train(npairs=128, steps=600)
    assert rep["pairs"] == 128
    assert rep["loss_last"] < rep["loss_first"] < 0  # A-cosine loss: more negative is better
    assert rep["val_plain_iters"] > 0 and rep["val_learned_iters"] > 0
    mm.rhs()
    plain = mm.solve(precond="bj3", stop_crit=1e-12)
    x_plain = mm.solution()
    learned = mm.solve(precond="learned", stop_crit=1e-12)
    x_learned = mm.solution()
    assert plain["converged"] and learned["converged"]
    assert _rel(x_learned, x_plain, npix) < 1e-4
    if not rep["enabled"]:
        # the network lost on validation: the learned mode is plain PCG
        assert learned["fallback_iter"] == 0 and learned["iterations"] == plain["iterations"]
    # the network forced on: flexible PCG with the correction still reaches the
    # same map; the iteration counts are what the network gains (or loses)
    rep_f = mm.learn_train(npairs=128, steps=600, force=True)
    assert rep_f["enabled"] == 1
    mm.rhs()
    forced = mm.solve(precond="learned", stop_crit=1e-12, maxiter=1000)
    assert forced["converged"] and forced["fallback_iter"] == -1
    assert _rel(mm.solution(), x_plain, npix) < 1e-4
    print(f"\nvalidation: plain {rep['val_plain_iters']} it {rep['val_plain_ms']:.1f} ms, "
          f"learned {rep['val_learned_iters']} it {rep['val_learned_ms']:.1f} ms, "
          f"enabled {rep['enabled']}; solve: plain {plain['iterations']}, "
          f"learned mode {learned['iterations']}, network forced {forced['iterations']}")
