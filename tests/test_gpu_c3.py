"""The ACA configuration (Matern nu = 3/2, range 0.05, ACA tol 1e-8, LogLevel(8), 8 right-hand
sides) checked against dense linear algebra.

* Dense subsample: at n = 2^14 with the configuration's nugget 1e-4 the compressed matrix
  factorises; its logdet and solves are compared with the dense Cholesky factorisation of the
  exact kernel matrix (FP64 on the GPU through torch, the checker here).  The gap is the ACA
  compression error (tol 1e-8 relative per block, amplified by the conditioning the small nugget
  gives), not the factorisation's: the solve of the compressed matrix itself has an FP64-level
  residual.
* n = 2^18 with nugget 1e-4: the factorisation raises PosDefException.  The compressed matrix
  is itself indefinite, shown without the factorisation: its principal submatrix on the 4096
  points of each half closest to the top-level split (columns of the compressed matrix from
  the pre-factorisation matvec, baseoverloads.jl:152-169) has a negative eigenvalue, and by
  eigenvalue interlacing so has the whole matrix.  No symmetric factorisation of it (the
  reference's symmetricfactorize!, symfact.jl:6-49, included) can succeed.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PARAMS = (1.0, 0.05, 1e-4)


def dense_matern(torch, pts, params):
    """Matern nu = 3/2 kernel matrix plus the nugget on the diagonal, FP64 on the GPU."""
    x = torch.as_tensor(pts, dtype=torch.float64, device="cuda")
    d = torch.cdist(x, x)
    z = (3.0 ** 0.5) * d / params[1]
    k = params[0] * (1.0 + z) * torch.exp(-z)
    k.diagonal().add_(params[2])
    return k


def test_c3_dense_subsample_2p14(lib):
    torch = pytest.importorskip("torch")
    import kmhodlr as K
    from kmhodlr.data import uniform_points
    n = 2 ** 14
    pts = uniform_points(n, 20260401)
    rhs = np.asfortranarray(np.random.default_rng(20260402).standard_normal((n, 8)))
    hk = K.KernelHODLR(K.KernelMatrix(pts, pts, PARAMS, K.Matern32()), 1e-8, 0, K.LogLevel(8), nystrom=False)
    y_h = hk @ rhs
    K.symmetricfactorize(hk)
    x_h = hk.ldiv(rhs)
    ld_h = hk.logdet()
    kd = dense_matern(torch, pts, PARAMS)
    b = torch.as_tensor(rhs, device="cuda")
    # the compressed matrix's own solve: residual at FP64 level through its matvec
    res = np.linalg.norm(hk @ x_h - rhs) / np.linalg.norm(rhs)
    assert res < 1e-10
    # compression error of the matvec, and the dense Cholesky comparison
    y_d = (kd @ b).cpu().numpy()
    mv_err = np.linalg.norm(y_h - y_d) / np.linalg.norm(y_d)
    L = torch.linalg.cholesky(kd)
    ld_d = float(2.0 * torch.log(torch.diagonal(L)).sum())
    x_d = torch.cholesky_solve(b, L).cpu().numpy()
    x_err = np.linalg.norm(x_h - x_d) / np.linalg.norm(x_d)
    res_d = float(torch.linalg.norm(kd @ torch.as_tensor(x_h, device="cuda") - b) / torch.linalg.norm(b))
    print(f"n=2^14: matvec {mv_err:.2e}, logdet {ld_h:.10f} vs {ld_d:.10f} ({abs(ld_h - ld_d):.2e}), "
          f"solve {x_err:.2e}, exact-K residual {res_d:.2e}")
    # measured: matvec 8.1e-8, logdet 2.6e-4 absolute (3e-9 relative), solve 7.1e-5 and exact-K
    # residual 3.0e-4 (the 1e-8 block tolerance amplified by cond(K) ~ 1e4 from the 1e-4 nugget)
    assert mv_err < 1e-6
    assert abs(ld_h - ld_d) < 1e-2
    assert x_err < 1e-3
    assert res_d < 3e-3


def test_c3_nugget_1e4_compressed_matrix_indefinite(lib):
    torch = pytest.importorskip("torch")
    import kmhodlr as K
    from kmhodlr.data import uniform_points
    n = 2 ** 18
    pts = uniform_points(n, 20260403)
    hk = K.KernelHODLR(K.KernelMatrix(pts, pts, PARAMS, K.Matern32()), 1e-8, 0, K.LogLevel(8), nystrom=False)
    # the top-level split of the k-d ordered points: the axis that separates the two halves
    h = n // 2
    a, c = pts[:h], pts[h:]
    ax = 0 if a[:, 0].max() <= c[:, 0].min() else 1
    assert a[:, ax].max() <= c[:, ax].min()
    cut = 0.5 * (a[:, ax].max() + c[:, ax].min())
    sa = np.argsort(cut - a[:, ax])[:4096]
    sc = h + np.argsort(c[:, ax] - cut)[:4096]
    S = np.sort(np.concatenate([sa, sc]))
    # columns S of the compressed matrix, 256 at a time
    cols = []
    for q in range(0, S.size, 256):
        X = np.zeros((n, 256), order="F")
        blk = S[q:q + 256]
        X[blk, np.arange(blk.size)] = 1.0
        cols.append((hk @ X)[S, :blk.size])
    H = np.concatenate(cols, axis=1)
    assert np.max(np.abs(H - H.T)) < 1e-10 * np.max(np.abs(H))
    Ht = torch.as_tensor(0.5 * (H + H.T), device="cuda")
    lam_h = float(torch.linalg.eigvalsh(Ht)[0])
    kd = dense_matern(torch, pts[S], PARAMS)
    lam_k = float(torch.linalg.eigvalsh(kd)[0])
    err = float(torch.linalg.matrix_norm(Ht - kd, ord=2))
    print(f"n=2^18, nugget 1e-4: lambda_min compressed {lam_h:.3e}, exact {lam_k:.3e}, "
          f"||HK - K|| on the subset {err:.3e}")
    assert lam_k > 0.0
    assert lam_h < 0.0
    with pytest.raises(K.PosDefException):
        K.symmetricfactorize(hk)
