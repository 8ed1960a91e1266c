"""The recurrences of the exact J v Arnoldi body (delayed one-reduction CGS2, krylov.cuh
k_gmres_prim_z / k_gmres_gather_dot) restated in numpy on the host: from one set of dots
per iteration (of the stored vectors with the pending vector and with the product, and
|w|^2) they must give the Arnoldi basis and Hessenberg matrix of plain modified
Gram-Schmidt, including when the pending vector is scaled by 1/|w| (its first-pass vector
times lam) and the column divides lam out.  Host logic only: the GPU kernels are checked
against the host-driven Gram-Schmidt loop in test_gpu_krylov.py."""
import numpy as np
import pytest


def mgs_arnoldi(A, b, m):
    n = b.size
    V = np.zeros((n, m + 1))
    H = np.zeros((m + 1, m))
    V[:, 0] = b / np.linalg.norm(b)
    for j in range(m):
        w = A @ V[:, j]
        for i in range(j + 1):
            H[i, j] = V[:, i] @ w
            w -= H[i, j] * V[:, i]
        H[j + 1, j] = np.linalg.norm(w)
        V[:, j + 1] = w / H[j + 1, j]
    return V, H


def dcgs2_arnoldi(A, b, m, scale_by_w=True):
    """The kernels' recurrences.  Slots hold the stored (unnormalised) basis vectors u_k
    with v_k = sc_k u_k, and the pending vector P_j; the product at iteration j is
    w = A (sig_j P_j); one reduction gives <u_k, P_j>, <u_k, w> (k <= j, u_j := P_j) and
    |w|^2."""
    n = b.size
    slots = np.zeros((n, m + 1))
    sc = np.ones(m + 1)
    sig = np.ones(m + 2)
    ilam = np.ones(m + 2)
    Hu = np.zeros((m + 1, m))
    h1 = np.zeros(m + 1)
    slots[:, 0] = b / np.linalg.norm(b)           # P_0 = V_0 (k_gmres_start)
    for jn in range(m + 2):
        if jn > 0:
            j = jn - 1
            P, wv = slots[:, j].copy(), w
            dp = slots[:, :j + 1].T @ P              # gather kernel: dots with P_j
            dw = slots[:, :j + 1].T @ wv             # ... with w
            wsq = wv @ wv                            # ... and |w|^2
            s = sc[:j] * sig[j] * dp[:j]
            g = np.empty(j + 1)
            g[:j] = sc[:j] * dw[:j]
            if j > 0:
                beta = np.sqrt(max(sig[j] ** 2 * dp[j] - s @ s, 0.0))
                r = 1.0 / beta
            else:
                beta, r = 1.0, 1.0
            g[j] = (sig[j] * dw[j] - s @ g[:j]) * r
            scj = sig[j] * r
            u = P - slots[:, :j] @ (sc[:j] ** 2 * dp[:j])     # V_j (slot j)
            slots[:, j] = u
            Pn = wv - slots[:, :j] @ (g[:j] * sc[:j]) - g[j] * scj * u
            sgn = 1.0 / np.sqrt(wsq) if scale_by_w else r
            # Givens block: column j - 1 final, then column j's first-pass entries
            if j > 0:
                c = j - 1
                Hu[:c + 1, c] = h1[:c + 1] + s * ilam[j]
                Hu[c + 1, c] = beta * ilam[j]
            if j < m:
                hs = Hu[:j + 1, :j] @ s if j > 0 else np.zeros(1)
                h1[:j + 1] = (g - hs) * r
            sc[j] = scj
            sig[jn] = sgn
            ilam[jn] = r / sgn                       # 1/lam_jn = r |w|
            if jn > m:
                break
            slots[:, jn] = Pn
        else:
            pass
        if jn <= m:
            w = A @ (sig[jn] * slots[:, jn])         # the product of iteration jn
    V = slots[:, :m] * sc[:m]
    return V, Hu


@pytest.mark.parametrize("scale_by_w", [True, False])
@pytest.mark.parametrize("n,m,seed", [(60, 12, 0), (200, 30, 1)])
def test_dcgs2_recurrences_reproduce_arnoldi(n, m, seed, scale_by_w):
    rng = np.random.default_rng(seed)
    A = np.eye(n) * 3.0 + rng.standard_normal((n, n)) / np.sqrt(n)
    b = rng.standard_normal(n)
    V0, H0 = mgs_arnoldi(A, b, m)
    V1, H1 = dcgs2_arnoldi(A, b, m, scale_by_w)
    # an orthonormal basis and the Arnoldi relation A V = V H over the finished columns
    np.testing.assert_allclose(V1.T @ V1, np.eye(m), atol=1e-12)
    np.testing.assert_allclose(A @ V1[:, :m - 1], V1 @ H1[:m, :m - 1], atol=1e-12)
    # the same basis and Hessenberg matrix as modified Gram-Schmidt over the first columns
    # (later the Krylov space of this matrix is nearly invariant and any two orthogonal-
    # isation orders drift apart from their rounding, by ~30x per five columns)
    k = min(m, 12)
    np.testing.assert_allclose(H1[:k + 1, :k], H0[:k + 1, :k], rtol=0, atol=1e-8 * np.abs(H0).max())
    np.testing.assert_allclose(np.abs(V1[:, :k].T @ V0[:, :k]), np.eye(k), atol=1e-8)


def test_scaled_input_keeps_the_product_bounded():
    """With the input scaled by 1/|w| every product's input has norm <= 1 (the reason for
    the scale: the dots of an FP32 reduction stay in range), while the unscaled pending
    vector grows with |A|."""
    rng = np.random.default_rng(5)
    n, m = 80, 10
    A = (np.eye(n) + rng.standard_normal((n, n)) / np.sqrt(n)) * 1e6
    b = rng.standard_normal(n)
    norms = {}
    # the first pending vector after V_0: P_1 = w - g v_0 with w = A v_0
    v0 = b / np.linalg.norm(b)
    w0 = A @ v0
    P1 = w0 - (v0 @ w0) * v0
    norms[True] = np.linalg.norm(P1 / np.linalg.norm(w0))
    norms[False] = np.linalg.norm(P1)
    assert norms[True] <= 1.0
    assert norms[False] > 1e5
