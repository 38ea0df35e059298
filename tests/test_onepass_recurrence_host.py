"""The one-pass iteration form of the batched mixed-precision solver, restated
on the host in FP64 (numpy): the state the kernel carries between sweeps
(r and z of the previous sweep, the pending step nu, the next mu, the
direction p_old) and its finaliser's rules, against the textbook CG
recurrence that CGSolveQ follows (main/phys.c:2478-2525; nu = alpha / p.z,
mu = alpha_new / alpha_old).

Checked: the same iterates and the same iteration count at the stopping rule
sqrt(eps/eps0) < tol, also when reliable updates replace the residual by
b - A x and the sweep after each refresh re-forms its direction from it (the
rollback the kernel does: the refreshed residual is written where the next
sweep reads r, the pending step is dropped, mu = rho_true / rho_prev).
CPU only."""
import numpy as np


def laplacian_2d(n, shift=0.05, seed=0):
    """SPD test matrix: a 5-point Laplacian on an n x n grid with a random
    positive diagonal shift (like the pressure operator: symmetric, stiff)."""
    rng = np.random.default_rng(seed)
    N = n * n
    A = np.zeros((N, N))
    for i in range(n):
        for j in range(n):
            u = i * n + j
            A[u, u] = 4.0 + shift * rng.random()
            for di, dj in ((1, 0), (-1, 0), (0, 1), (0, -1)):
                a, b = i + di, j + dj
                if 0 <= a < n and 0 <= b < n:
                    A[u, a * n + b] = -1.0
    return A


def cg_reference(A, b, x0, tol, maxiters):
    """CG as CGSolveQ runs it with qprecond 1 (the scaled system, s = r)."""
    x = x0.copy()
    r = b - A @ x
    p = r.copy()
    alpha = r @ r
    eps0 = alpha
    xs = []
    n = 0
    while n < maxiters:
        z = A @ p
        nu = alpha / (p @ z)
        x = x + nu * p
        r = r - nu * z
        alpha_new = r @ r
        n += 1
        xs.append(x.copy())
        if np.sqrt(alpha_new / eps0) < tol:
            break
        p = r + (alpha_new / alpha) * p
        alpha = alpha_new
    return x, n, xs


def cg_one_pass(A, b, x0, tol, maxiters, refresh_every=None):
    """The kernel's one-pass form: each sweep takes the pending step
    (r -= nu z, x += nu p_old), forms p = r + mu p_old and z = A p, and sums
    p.z, r.r, r.z, z.z; the finaliser sets nu = r.r / p.z and the next
    mu = (r.r - 2 nu r.z + nu^2 z.z) / r.r.  refresh_every: flag a reliable
    update every that many counted iterations (the kernel flags on a residual
    drop; the rollback is the same)."""
    x = x0.copy()
    r = b - A @ x
    z = np.zeros_like(r)
    p_old = np.zeros_like(r)
    nu, mu = 0.0, 0.0
    rho_prev = r @ r
    eps0 = rho_prev
    n = 0
    xs = []
    last_refresh = 0
    for _ in range(4 * maxiters + 8):
        moved = nu != 0.0
        r_new = r - nu * z
        x = x + nu * p_old
        p = r_new + mu * p_old
        z_new = A @ p
        pz, rr, rz, zz = p @ z_new, r_new @ r_new, r_new @ z_new, z_new @ z_new
        if moved:
            n += 1
            xs.append(x.copy())
            if np.sqrt(rr / eps0) < tol or n >= maxiters:
                return x, n, xs
            if refresh_every and n - last_refresh >= refresh_every:
                # reliable update: true residual in place of this sweep's r;
                # this sweep's p and z are dropped (p_old, r's buffer kept)
                last_refresh = n
                r = b - A @ x
                rho_true = r @ r
                mu = rho_true / rho_prev
                nu = 0.0
                continue
        nu_j = rr / pz
        rnext = rr - 2.0 * nu_j * rz + nu_j * nu_j * zz
        mu = max(rnext, 0.0) / rr
        nu = nu_j
        rho_prev = rr
        r, z, p_old = r_new, z_new, p
    raise AssertionError("no convergence")


def test_one_pass_form_follows_the_reference_recurrence():
    A = laplacian_2d(12)
    rng = np.random.default_rng(1)
    b = rng.standard_normal(A.shape[0])
    x0 = 0.01 * rng.standard_normal(A.shape[0])
    x_ref, n_ref, xs_ref = cg_reference(A, b, x0, 1e-10, 2000)
    x_one, n_one, xs_one = cg_one_pass(A, b, x0, 1e-10, 2000)
    assert n_one == n_ref
    scale = np.linalg.norm(x_ref)
    # every iterate agrees to rounding (the recurrences differ only in how
    # the next residual norm is obtained)
    for a, c in zip(xs_one, xs_ref):
        assert np.linalg.norm(a - c) <= 1e-9 * scale
    assert np.linalg.norm(A @ x_one - b) <= 1e-9 * np.linalg.norm(b)


def test_one_pass_refresh_rollback_keeps_convergence():
    """With reliable updates every 15 iterations the one-pass form still meets
    the stopping rule on the true residual within a few iterations of the
    reference count, and its solution agrees with the reference's."""
    A = laplacian_2d(12, seed=3)
    rng = np.random.default_rng(2)
    b = rng.standard_normal(A.shape[0])
    x0 = np.zeros(A.shape[0])
    x_ref, n_ref, _ = cg_reference(A, b, x0, 1e-10, 2000)
    x_one, n_one, _ = cg_one_pass(A, b, x0, 1e-10, 2000, refresh_every=15)
    assert abs(n_one - n_ref) <= max(3, n_ref // 20), (n_one, n_ref)
    assert np.linalg.norm(b - A @ x_one) <= 1e-9 * np.linalg.norm(b)
    assert np.linalg.norm(x_one - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
