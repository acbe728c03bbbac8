"""The FP64 oracles on known answers (CPU only)."""
import numpy as np
import scipy.linalg


def test_largest_eigenvalue_agrees_with_lapack(port):
    rng = np.random.default_rng(1)
    m = rng.normal(size=(2000, 3, 3))
    s = np.einsum("nij,nkj->nik", m, m)
    got = port.largest_eigenvalue(s.reshape(-1, 9))
    assert np.allclose(got, np.linalg.eigvalsh(s)[:, -1], rtol=1e-12, atol=1e-12)
    # repeated eigenvalues and diagonal matrices
    d = np.diag([2.0, 2.0, 2.0]).reshape(1, 9)
    assert port.largest_eigenvalue(d)[0] == 2.0
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    a = q @ np.diag([5.0, 5.0, 1.0]) @ q.T
    assert abs(port.largest_eigenvalue(a.reshape(1, 9))[0] - 5.0) < 1e-12
    # the trigonometric closed form (cross-check): loses accuracy only near a
    # repeated largest eigenvalue, and stays far inside the FTLE bar there
    closed = port.largest_eigenvalue(s.reshape(-1, 9), closed_form=True)
    assert np.allclose(closed, got, rtol=1e-10)
    assert abs(port.largest_eigenvalue(a.reshape(1, 9), closed_form=True)[0] - 5.0) < 1e-7


def test_uniform_field_with_dyadic_step_is_exact(port):
    from pars_gb300 import workloads as W
    f = W.uniform_field(16, (0.5, 0.25, -0.125), spacing=0.25)
    start = np.array([[1.0, 1.0, 3.0]])
    end, steps, _ = port.advect_fp64(f, start, 16, integrator=2, mode=1, step=0.125)
    assert steps[0] == 16
    assert np.array_equal(end[0], start[0] + 16 * 0.125 * np.array([0.5, 0.25, -0.125]))


def test_linear_field_rk4_matches_matrix_exponential(port):
    from pars_gb300 import workloads as W
    A = np.array([[0.2, 0.1, 0.0], [-0.1, 0.1, 0.05], [0.0, 0.02, -0.3]])
    n, h = 33, 0.1
    f = W.linear_field(n, A, spacing=h)
    c = h * (n - 1) / 2
    start = np.array([[c + 0.1, c - 0.2, c + 0.05]])
    T, dt = 2.0, 0.01
    end, steps, _ = port.advect_fp64(f, start, int(round(T / dt)), integrator=2, mode=1, step=dt)
    exact = scipy.linalg.expm(A * T) @ (start[0] - c) + c
    # the grid samples are FP32, so agreement is to FP32 rounding of the field
    assert np.linalg.norm(end[0] - exact) < 1e-5


def test_ftle_fp64_of_linear_flow_map(port):
    A = np.array([[0.3, 0.05, 0.0], [0.02, -0.1, 0.04], [0.0, 0.03, -0.2]])
    T = 2.0
    M = scipy.linalg.expm(A * T)
    n, h = 9, 0.1
    g = np.stack(np.meshgrid(*[np.arange(n) * h] * 3, indexing="ij"), -1)
    flow = (g @ M.T).astype(np.float32)
    ftle = port.ftle_fp64(flow, np.full(3, h, np.float32), T)
    expected = np.log(np.linalg.svd(M, compute_uv=False).max()) / T
    assert np.abs(ftle[2:-2, 2:-2, 2:-2] - expected).max() < 1e-5


def test_fractional_anisotropy_fp64_of_linear_flow_map(port):
    """FA mode (ftle_map_generator.cpp:51-54) on phi(x) = M x: central
    differences give J = M exactly, so FA is that of the eigenvalues of M^T M."""
    A = np.array([[0.3, 0.05, 0.0], [0.02, -0.1, 0.04], [0.0, 0.03, -0.2]])
    M = scipy.linalg.expm(A * 2.0)
    n, h = 9, 0.1
    g = np.stack(np.meshgrid(*[np.arange(n) * h] * 3, indexing="ij"), -1)
    flow = (g @ M.T).astype(np.float32)
    fa = port.ftle_fp64(flow, np.full(3, h, np.float32), 2.0, mode=1)
    l = np.linalg.eigvalsh(M.T @ M)
    expected = np.sqrt(0.5) * np.sqrt((l[0] - l[1]) ** 2 + (l[1] - l[2]) ** 2 + (l[2] - l[0]) ** 2) / np.sqrt((l ** 2).sum())
    # FP32 flow-map samples limit the agreement
    assert np.abs(fa[2:-2, 2:-2, 2:-2] - expected).max() < 1e-5
    # an isotropic map (phi = 2 x): C = 4 I, anisotropy 0
    iso = port.ftle_fp64((2 * g).astype(np.float32), np.full(3, h, np.float32), 2.0, mode=1)
    assert np.abs(iso).max() < 1e-6


def test_every_integrator_has_its_order_on_an_exact_linear_field(port):
    """The FP64 oracle's re-sampled schemes (the true forms of integrators.hpp:
    16-23) on v = A (x - c) with dyadic A, grid and centre, which trilinear
    interpolation reproduces exactly: halving h divides the error by 2^p,
    p = 1 (Euler), 2 (modified midpoint, Adams-Bashforth 2, Adams-Bashforth-
    Moulton 2), 4 (RK4), 5 (Cash-Karp, Dormand-Prince), >= 6.5 for
    Fehlberg 7(8) before FP64 rounding takes over."""
    from pars_gb300 import workloads as W
    A = np.array([[0.25, 0.5, 0.0], [-0.5, 0.25, 0.125], [0.0, -0.125, -0.25]])
    n, sp = 33, 0.25
    f = W.linear_field(n, A, spacing=sp)
    c = sp * (n - 1) / 2
    start = np.array([[c + 0.5, c - 0.75, c + 0.25]])
    T = 2.0
    exact = scipy.linalg.expm(A * T) @ (start[0] - c) + c
    orders = [1, 2, 4, 5, 5, 6.5, 2, 2]
    for k, p in enumerate(orders):
        hs = (0.5, 0.25) if k == 5 else (0.25, 0.125)
        errs = []
        for h in hs:
            end, _, _ = port.advect_fp64(f, start, int(round(T / h)), integrator=k, mode=1, step=h)
            errs.append(np.linalg.norm(end[0] - exact))
        assert np.log2(errs[0] / errs[1]) >= p - 0.3, (k, errs)
