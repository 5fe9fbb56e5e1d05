"""CPU oracle of the learned proposal's network (test infrastructure only: tests/, smoke() and bench.py's
CPU leg compare the GPU network with it; the product path never imports it).

The network and its training objective have no counterpart in the reference (they are the learned
proposal that the plain MC_move_rototranslate, MC.c:311-340, falls back to). This module restates them
in numpy so that the tensor-core kernels can be checked:

* forward(): z = W3 relu(W2 relu(W1 x + b1) + b2) + b3 with the operand roundings of the GPU path -- x,
  weights and hidden activations rounded to BF16 (round to nearest even), products accumulated in
  float64 here (FP32 in tensor memory there), biases added in FP32;
* grad(): the gradient of L = -(1/n) sum J, J = sum_k pi_k u_k + tau H(softmax z), pi = (1 - floor)
  softmax(z) + floor e_0, back-propagated with the same BF16 roundings of dZ, dA2 and dA1 that the GPU
  feeds to its tensor-core GEMMs (bias gradients = column sums of those rounded values);
* grad_exact(): the same gradient in float64 without any rounding (checked against finite differences).
"""
import numpy as np

IN, HID, OUT = 36, 64, 4
OFF_W1 = 0
OFF_B1 = OFF_W1 + HID * IN
OFF_W2 = OFF_B1 + HID
OFF_B2 = OFF_W2 + HID * HID
OFF_W3 = OFF_B2 + HID
OFF_B3 = OFF_W3 + OUT * HID
NPARAMS = OFF_B3 + OUT
SAMPLE = IN + OUT


def bf16(x):
    """FP32 -> BF16 (round to nearest, ties to even), returned as float32 values."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).reshape(x.shape)


def unpack(P):
    P = np.asarray(P, dtype=np.float32)
    return (P[OFF_W1:OFF_B1].reshape(HID, IN), P[OFF_B1:OFF_W2], P[OFF_W2:OFF_B2].reshape(HID, HID), P[OFF_B2:OFF_W3],
            P[OFF_W3:OFF_B3].reshape(OUT, HID), P[OFF_B3:NPARAMS])


def pack(W1, b1, W2, b2, W3, b3):
    return np.concatenate([np.ravel(a).astype(np.float32) for a in (W1, b1, W2, b2, W3, b3)])


def init_params(seed=0, out_scale=0.0):
    """Uniform fan-in initialisation of the hidden layers; the output layer starts at out_scale (0: the
    uniform mixture)."""
    rng = np.random.default_rng(seed)
    W1 = rng.uniform(-1, 1, (HID, IN)) * np.sqrt(6.0 / IN)
    W2 = rng.uniform(-1, 1, (HID, HID)) * np.sqrt(6.0 / HID)
    W3 = rng.uniform(-1, 1, (OUT, HID)) * out_scale
    return pack(W1, np.zeros(HID), W2, np.zeros(HID), W3, np.zeros(OUT))


def _mm(a, b):
    return (a.astype(np.float64) @ b.astype(np.float64)).astype(np.float32)


def forward(P, X, full=False):
    W1, b1, W2, b2, W3, b3 = unpack(P)
    Xb = bf16(np.asarray(X, dtype=np.float32).reshape(-1, IN))
    a1 = _mm(Xb, bf16(W1).T) + b1
    h1 = bf16(np.maximum(a1, 0))
    a2 = _mm(h1, bf16(W2).T) + b2
    h2 = bf16(np.maximum(a2, 0))
    z = _mm(h2, bf16(W3).T) + b3
    if full:
        return z, (Xb, a1, h1, a2, h2)
    return z


def mixture(z, floor):
    """Mixture weights pi = (1 - floor) softmax(z) + floor e_0 (float64)."""
    z = np.asarray(z, dtype=np.float64)
    e = np.exp(z - z.max(axis=1, keepdims=True))
    s = e / e.sum(axis=1, keepdims=True)
    pi = (1 - floor) * s
    pi[:, 0] += floor
    return pi


def objective_grad_z(z, u, floor, tau):
    """(J per sample, dJ/dz per sample), float64."""
    z = np.asarray(z, dtype=np.float64)
    u = np.asarray(u, dtype=np.float64)
    m = z.max(axis=1, keepdims=True)
    e = np.exp(z - m)
    S = e.sum(axis=1, keepdims=True)
    s = e / S
    ls = (z - m) - np.log(S)
    H = -(s * ls).sum(axis=1, keepdims=True)
    ub = (s * u).sum(axis=1, keepdims=True)
    pi = (1 - floor) * s
    pi[:, 0] += floor
    J = (pi * u).sum(axis=1) + tau * H[:, 0]
    g = (1 - floor) * s * (u - ub) - tau * s * (ls + H)
    return J, g


def grad(P, samples, floor, tau):
    """Gradient with the GPU's operand roundings: (grad[NPARAMS] float64, mean J)."""
    S = np.asarray(samples, dtype=np.float32).reshape(-1, SAMPLE)
    n = S.shape[0]
    X, U = S[:, :IN], S[:, IN:]
    W1, b1, W2, b2, W3, b3 = unpack(P)
    z, (Xb, a1, h1, a2, h2) = forward(P, X, full=True)
    J, g = objective_grad_z(z, U, floor, tau)
    dz = bf16((-g / n).astype(np.float32))
    dH2 = _mm(dz, bf16(W3))
    dA2 = bf16(np.where(a2 > 0, dH2, 0).astype(np.float32))
    dH1 = _mm(dA2, bf16(W2))
    dA1 = bf16(np.where(a1 > 0, dH1, 0).astype(np.float32))
    f = lambda a, b: a.astype(np.float64).T @ b.astype(np.float64)
    G = np.concatenate([f(dA1, Xb).ravel(), dA1.astype(np.float64).sum(0), f(dA2, h1).ravel(), dA2.astype(np.float64).sum(0),
                        f(dz, h2).ravel(), dz.astype(np.float64).sum(0)])
    return G, float(J.mean())


def loss_exact(P, samples, floor, tau):
    """L = -(1/n) sum J in float64, no rounding."""
    S = np.asarray(samples, dtype=np.float64).reshape(-1, SAMPLE)
    W1, b1, W2, b2, W3, b3 = _unpack64(P)
    X, U = S[:, :IN], S[:, IN:]
    a1 = X @ W1.T + b1
    a2 = np.maximum(a1, 0) @ W2.T + b2
    z = np.maximum(a2, 0) @ W3.T + b3
    J, _ = objective_grad_z(z, U, floor, tau)
    return -J.mean()


def _unpack64(P):
    P = np.asarray(P, dtype=np.float64)
    return (P[OFF_W1:OFF_B1].reshape(HID, IN), P[OFF_B1:OFF_W2], P[OFF_W2:OFF_B2].reshape(HID, HID), P[OFF_B2:OFF_W3],
            P[OFF_W3:OFF_B3].reshape(OUT, HID), P[OFF_B3:NPARAMS])


def grad_exact(P, samples, floor, tau):
    """dL/dP in float64 without rounding (the formulas grad() rounds)."""
    S = np.asarray(samples, dtype=np.float64).reshape(-1, SAMPLE)
    n = S.shape[0]
    W1, b1, W2, b2, W3, b3 = _unpack64(P)
    X, U = S[:, :IN], S[:, IN:]
    a1 = X @ W1.T + b1
    h1 = np.maximum(a1, 0)
    a2 = h1 @ W2.T + b2
    h2 = np.maximum(a2, 0)
    z = h2 @ W3.T + b3
    _, g = objective_grad_z(z, U, floor, tau)
    dz = -g / n
    dA2 = (dz @ W3) * (a2 > 0)
    dA1 = (dA2 @ W2) * (a1 > 0)
    return np.concatenate([(dA1.T @ X).ravel(), dA1.sum(0), (dA2.T @ h1).ravel(), dA2.sum(0), (dz.T @ h2).ravel(), dz.sum(0)])


def random_samples(n, seed=0):
    """Synthetic training samples: features like patch-site vectors (|v| <~ 1.6), utilities in [0, 3)."""
    rng = np.random.default_rng(seed)
    X = rng.uniform(-1.6, 1.6, (n, IN)).astype(np.float32)
    X[rng.random((n, IN)) < 0.3] = 0.0  # zero padding of absent neighbours
    U = rng.uniform(0, 3, (n, OUT)).astype(np.float32)
    return np.concatenate([X, U], axis=1)


# ---------------------------------------------------------------- features of the learned proposal
def base_patches():
    """The four tetrahedral patch directions as the reference builds them (system.c:20-31): +-0.5/sqrt(3)
    components, each vector then normalised."""
    h = 0.5 / np.sqrt(3.0)
    v = np.array([[-h, -h, h], [h, -h, -h], [h, h, h], [-h, h, -h]], dtype=np.float64)
    for i in range(4):
        n = np.sqrt((v[i, 0] * v[i, 0] + v[i, 1] * v[i, 1]) + v[i, 2] * v[i, 2])
        v[i] = v[i] / n
    return v


def canonical_image(r, R, box):
    """FP32 image of the canonical state as the engine forms it: the position wrapped into the box with an
    FP32 guess of the image index (x - k L in float64, k = floor(fl(x) / fl(L)) in float32) and rounded to
    FP32; the orientation rows rounded to FP32 (the engine evaluates R0 . Q(q) in FP32, which equals the
    rounded R while q is the identity -- right after an upload)."""
    r = np.asarray(r, dtype=np.float64).reshape(-1, 3)
    box = np.asarray(box, dtype=np.float64)
    Lf = box.astype(np.float32)
    k = np.floor(r.astype(np.float32) * (np.float32(1.0) / Lf)).astype(np.float64)
    y = r - k * box
    return y.astype(np.float32), np.asarray(R, dtype=np.float64).reshape(-1, 3, 3).astype(np.float32)


def features(r, R, box, kf_delta, nb=3):
    """features[N][36] of every particle: patch sites (centre + 0.5 patch direction) of its `nb` nearest
    neighbours within (1 + delta) sqrt(1 - 1e-4), nearest first (ties by index), minimum image, in the
    particle's frame (R^T . site), zero-padded. FP32 arithmetic operation by operation, as the engine."""
    pos, Rf = canonical_image(r, R, box)
    N = pos.shape[0]
    L = np.asarray(box, dtype=np.float64).astype(np.float32)
    iL = np.float32(1.0) / L
    rf2 = np.float32(np.float32((1.0 + kf_delta) * (1.0 + kf_delta)) * np.float32(0.9999))
    b32 = base_patches().astype(np.float32)
    half = np.float32(0.5)
    out = np.zeros((N, 12 * nb), dtype=np.float32)
    for i in range(N):
        v = pos - pos[i]
        v = v - L * np.rint(v * iL)
        r2 = (v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2]
        r2[i] = np.float32(np.inf)
        cand = np.nonzero(r2 < rf2)[0]
        if cand.size == 0:
            continue
        order = cand[np.lexsort((cand, r2[cand]))][:nb]  # ties by particle index, as the engine
        Ri = Rf[i]
        for n, j in enumerate(order):
            dl = v[j]
            Rj = Rf[j]
            for m in range(4):
                p = (Rj[:, 0] * b32[m, 0] + Rj[:, 1] * b32[m, 1]) + Rj[:, 2] * b32[m, 2]
                site = dl + half * p
                f = (Ri[0, :] * site[0] + Ri[1, :] * site[1]) + Ri[2, :] * site[2]
                out[i, 12 * n + 3 * m:12 * n + 3 * m + 3] = f
    return out


def mixture_density_ratio(pi_new, pi_old, scale_disp, scale_theta, disp_max, theta_max, d, theta):
    """q(x' -> x) / q(x -> x') of one move (displacement d, angle theta) under the four-component mixture."""
    a = np.array([disp_max * s for s in scale_disp])
    t = np.minimum(np.array([theta_max * s for s in scale_theta]), np.pi)
    m = np.max(np.abs(d))
    c = np.where((m <= a / 2) & (theta < t), 1.0 / (a ** 3 * t), 0.0)
    return float(np.dot(pi_new, c) / np.dot(pi_old, c))
