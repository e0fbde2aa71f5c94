"""Oracle of the learned preconditioner's network (test infrastructure only).

The reference has no learned preconditioner; this restates the network that
yukawacolourednoise_gb300/csrc/yk_learned.cu implements, so that the CUDA
forward pass and its weight gradients can be checked (tests/test_learned.py),
and its own gradients are pinned against central finite differences.

Network (one real plane; the Dirac operator has real coefficients, so a
complex field is two independent real planes):
  * fields are channel-major arrays X[c, n], site n = t * Nx + x;
  * N: features F r = (r_0..r_3, sigma * r_0..sigma * r_3) (8 channels), then
    layers Y[o, n] = sum_k sum_i W_l[k, i, o] s_k(n) X[i, nb_k(n)] over the
    taps k = (dt + 1) * 3 + (dx + 1), dt, dx in {-1, 0, 1}, nb_k(n) the site
    at (t + dt mod Nt, x + dx mod Nx) and s_k(n) = -1 when t + dt wraps
    (antiperiodic in time, as the fermion fields), else +1; channels
    8 -> 8 -> ... -> 8 -> 4, no activation;
  * M(r) = skip r + N^T N r: symmetric positive definite; N^T runs the
    transposed layers in reverse order and ends with F^T (a, b) = a + sigma b.
Loss of a pair (r, e) (residual and error, A e = r, A = D^dag D): the energy
norm of the error left by the correction, (M r - e)^T A (M r - e) =
|D (M r - e)|^2 (the plain norm would be dominated by the smooth, low modes
of e).
"""
import numpy as np

TAPS = [(dt, dx) for dt in (-1, 0, 1) for dx in (-1, 0, 1)]


def shift(X, Nt, Nx, dt, dx):
    """S[c, n] = s(n) X[c, nb(n)] for the tap (dt, dx)."""
    C = X.shape[0]
    A = X.reshape(C, Nt, Nx)
    B = np.roll(A, shift=(-dt, -dx), axis=(1, 2)).copy()
    if dt == 1:
        B[:, Nt - 1, :] *= -1.0
    elif dt == -1:
        B[:, 0, :] *= -1.0
    return B.reshape(C, Nt * Nx)


def features(r, sigma):
    """F r: r (4, V), sigma (V,) -> (8, V)."""
    return np.concatenate([r, sigma[None, :] * r], axis=0)


def layer(X, W, Nt, Nx):
    """W: (9, Cin, Cout)."""
    Y = np.zeros((W.shape[2], X.shape[1]))
    for k, (dt, dx) in enumerate(TAPS):
        Y += W[k].T @ shift(X, Nt, Nx, dt, dx)
    return Y


def layer_T(Y, W, Nt, Nx):
    """The transpose of layer(): Cout -> Cin (the opposite tap, the same sign)."""
    X = np.zeros((W.shape[1], Y.shape[1]))
    for k, (dt, dx) in enumerate(TAPS):
        X += shift(W[k] @ Y, Nt, Nx, -dt, -dx)
    return X


def wgrad(X, Y, Nt, Nx):
    """d/dW of sum(Y * layer(X, W)): [k] = shift_k(X) @ Y^T."""
    return np.stack([shift(X, Nt, Nx, dt, dx) @ Y.T for dt, dx in TAPS])


def net_N(Ws, r, sigma, Nt, Nx):
    X = features(r, sigma)
    acts = [X]
    for W in Ws:
        X = layer(X, W, Nt, Nx)
        acts.append(X)
    return X, acts


def apply_M(Ws, r, sigma, Nt, Nx, skip):
    """z = skip r + N^T N r, with the activations of N and of N^T."""
    v, acts = net_N(Ws, r, sigma, Nt, Nx)
    L = len(Ws)
    decs = [None] * (L + 1)
    decs[L] = v
    for l in range(L - 1, -1, -1):
        decs[l] = layer_T(decs[l + 1], Ws[l], Nt, Nx)
    a = decs[0]
    z = a[:4] + sigma[None, :] * a[4:] + skip * r
    return z, acts, decs


def grad_M(Ws, acts, decs, gz, sigma, Nt, Nx):
    """Weight gradients of sum(gz * M(r))."""
    L = len(Ws)
    gWs = [np.zeros_like(W) for W in Ws]
    g = features(gz, sigma)               # through F^T
    for l in range(L):                     # through dec[l] = L_l^T dec[l + 1]
        gWs[l] += wgrad(g, decs[l + 1], Nt, Nx)
        g = layer(g, Ws[l], Nt, Nx)
    for l in range(L - 1, -1, -1):         # through N
        gWs[l] += wgrad(acts[l], g, Nt, Nx)
        g = layer_T(g, Ws[l], Nt, Nx)
    return gWs


def plain_loss_and_grad(Ws, r, e, sigma, Nt, Nx, skip=0.0):
    """|M r - e|^2 and its weight gradients (pins grad_M by finite differences)."""
    z, acts, decs = apply_M(Ws, r, sigma, Nt, Nx, skip)
    d = z - e
    return float(np.sum(d * d)), grad_M(Ws, acts, decs, 2.0 * d, sigma, Nt, Nx)


def dirac_real(Nt, Nx, act, sigma, X, dag):
    """D (or D^dag) of a real field X (4, V) through the FP64 oracle of D."""
    from oracle import oracle as O
    return np.real(O.dirac(Nt, Nx, act, sigma, X.T.astype(np.complex128), dag)).T


def energy_loss_and_grad(Ws, r, e, sigma, Nt, Nx, act, skip=0.0):
    """|D (M r - e)|^2 (unscaled) and its weight gradients."""
    z, acts, decs = apply_M(Ws, r, sigma, Nt, Nx, skip)
    Dd = dirac_real(Nt, Nx, act, sigma, z - e, False)
    gz = 2.0 * dirac_real(Nt, Nx, act, sigma, Dd, True)
    return float(np.sum(Dd * Dd)), grad_M(Ws, acts, decs, gz, sigma, Nt, Nx)


def flexible_pcg(apply_A, apply_M, b, tol, max_iter, polak_ribiere=True):
    """Preconditioned CG on A x = b (x0 = 0) with the preconditioner M, the
    recurrence of csrc/yk_learned.cu (pcg_dp_kernel, pcg_dq_kernel,
    pcg_xr_kernel, pcg_z_kernel) in FP64: alpha = <r, z> / <p, q>; beta =
    -<z', q> / <p, q> (Polak-Ribiere, polak_ribiere=True) or <r', z'> / <r, z>
    (classical).  Returns x, iterations, the |r|^2 history."""
    x = np.zeros_like(b)
    r = b.copy()
    z = apply_M(r)
    p = np.zeros_like(b)
    beta = 0.0
    rz = float(np.sum(r * z))
    hist = [float(np.sum(r * r))]
    stop2 = tol * tol * hist[0]
    it = 0
    while hist[-1] > stop2 and it < max_iter:
        p = z + beta * p
        q = apply_A(p)
        pq = float(np.sum(p * q))
        alpha = rz / pq
        x = x + alpha * p
        r = r - alpha * q
        z = apply_M(r)
        rz_new = float(np.sum(r * z))
        beta = -float(np.sum(z * q)) / pq if polak_ribiere else rz_new / rz
        rz = rz_new
        hist.append(float(np.sum(r * r)))
        it += 1
    return x, it, hist


def init_weights(hidden, layers, seed):
    """Deterministic small initial weights (the tests pass them to the GPU)."""
    rng = np.random.default_rng(seed)
    dims = [8] + [hidden] * (layers - 1) + [4]
    return [rng.normal(scale=1.0 / np.sqrt(9 * dims[l]), size=(9, dims[l], dims[l + 1]))
            for l in range(layers)]
