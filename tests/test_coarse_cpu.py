"""The coarse space's Rayleigh-Ritz step (host code of the library, no GPU)
against scipy's generalized symmetric eigensolver, and the resulting two-level
balancing preconditioner inside PCG on the oracle's FP64 operator."""
import numpy as np
import pytest
import scipy.linalg as sla

import oracle
import sanepic_gb300 as sg
from sanepic_gb300 import build, synth


@pytest.fixture(scope="module", autouse=True)
def _lib():
    build.build()


def _pencil(rng, n, m, dup=0):
    """H = V^T A V and G = V^T M^-1 V for random SPD A, M^-1 and m vectors V
    (the last `dup` of them repeating earlier ones: G rank-deficient)."""
    X = rng.normal(size=(n, n))
    A = X @ X.T / n + 0.05 * np.eye(n)
    Minv = np.diag(rng.uniform(0.5, 2.0, n))
    V = rng.normal(size=(n, m))
    if dup:
        V[:, m - dup:] = V[:, :dup]
    return V.T @ A @ V, V.T @ Minv @ V


@pytest.mark.parametrize("m,kc,dup", [(12, 4, 0), (40, 16, 0), (40, 8, 6), (64, 32, 0)])
def test_ritz_step_matches_scipy(m, kc, dup):
    rng = np.random.default_rng(m + kc + dup)
    H, G = _pencil(rng, 80, m, dup)
    C, einv, th = sg.coarse_from_gram(H, G, kc)
    k = th.size
    assert k == kc
    keep = m - dup
    # reference: the same pencil restricted to the independent vectors
    ref = sla.eigh(H[:keep, :keep], G[:keep, :keep], eigvals_only=True)
    np.testing.assert_allclose(th, ref[:k], rtol=1e-8)
    np.testing.assert_allclose(C.T @ G @ C, np.eye(k), atol=1e-8)
    E = C.T @ H @ C
    np.testing.assert_allclose(E, np.diag(th), atol=1e-8 * th.max())
    np.testing.assert_allclose(einv @ E, np.eye(k), atol=1e-7)


def test_ritz_step_rejects_empty_input():
    C, einv, th = sg.coarse_from_gram(np.zeros((4, 4)), np.zeros((4, 4)), 2)
    assert th.size == 0


def test_balancing_preconditioner_on_oracle_operator():
    """The library's recipe on the oracle's FP64 operator: residuals of plain
    block-Jacobi PCG on training skies, V = M r, Rayleigh-Ritz through
    sg_coarse_from_gram, then PCG with the balancing preconditioner on a
    held-out sky takes fewer iterations than block-Jacobi PCG and reaches the
    same map."""
    spec = synth.ProblemSpec("coarse_cpu", ndet=4, nside=16, nseg=6, ns=4096,
                             fknee_range=(0.05, 0.2), alpha_range=(1.0, 2.0), problem=33)
    prob = synth.make_problem(spec, with_tod=False)
    s = oracle.Setup(prob)
    n, npix = 3 * s.npix, s.npix
    mask = oracle.masked(s)
    Mb = s.block_jacobi().reshape(npix, 3, 3)

    def A(x):
        return np.where(mask, 0.0, s.apply(np.where(mask, 0.0, x)))

    def M(r):
        Z = np.einsum("pij,pj->pi", Mb, r.reshape(3, npix).T)
        return np.where(mask, 0.0, Z.T.reshape(-1))

    def rhs(seed):
        p2 = dict(prob)
        p2["sky"] = synth.make_sky(spec, seed=seed)
        b, _ = s.rhs(synth.make_tod(p2, noise_seed_base=seed))
        return np.where(mask, 0.0, b)

    def pcg(b, prec, tol=1e-6, keep=None):
        x = np.zeros(n)
        r = b.copy()
        z = prec(r)
        d = z.copy()
        dl = r @ z
        for it in range(1, 300):
            q = A(d)
            a = dl / (d @ q)
            x += a * d
            r -= a * q
            if keep is not None:
                keep.append(r.copy())
            if np.linalg.norm(r) <= tol * np.linalg.norm(b):
                return x, it
            z = prec(r)
            dn = r @ z
            d = z + dn / dl * d
            dl = dn
        return x, 300

    R = []
    for seed in (5000, 5001, 5002):
        pcg(rhs(seed), M, tol=1e-9, keep=R)
    R = np.array(R[:96])
    V = np.array([M(r) for r in R])
    W = np.array([A(v) for v in V])
    C, einv, th = sg.coarse_from_gram(V @ W.T, V @ R.T, 16)
    assert th.size == 16 and th[0] > 0
    U, AU = C.T @ V, C.T @ W

    def two_level(r):
        c = einv @ (U @ r)
        y = M(r - AU.T @ c)
        return y + U.T @ (c - einv @ (AU @ y))

    b = rhs(6000)
    x_p, it_p = pcg(b, M)
    x_c, it_c = pcg(b, two_level)
    print(f"\nblock-Jacobi PCG {it_p} iterations, two-level {it_c}")
    assert it_c < it_p
    d = x_c - x_p
    d[:npix] -= d[:npix].mean()
    assert np.linalg.norm(d) / np.linalg.norm(x_p) < 1e-4
