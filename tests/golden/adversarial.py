"""Adversarial guard-band configurations: isolated pairs whose r^2 or patch cosines sit within a few
ulp to a few 1e-5 of the thresholds sigma^2 = 1, (1 + delta)^2 and cosmax.

Deterministic (numpy seeded). Written as .rrr text with 17 significant digits so that the reference's
loader (system.c:213-243) and the engine's reader produce the same doubles; the loader re-normalises the
orientation rows, so the realised cosines differ from the intended ones only at the 1e-16 level.
"""
import numpy as np

BASE = np.array([[-1, -1, 1], [1, -1, -1], [1, 1, 1], [-1, 1, -1]], dtype=float) / np.sqrt(3.0)


def _rot_to(a, b):
    """rotation matrix taking unit vector a to unit vector b"""
    v = np.cross(a, b)
    c = float(np.dot(a, b))
    if c < -0.999999:
        # 180 degrees about any axis orthogonal to a
        axis = np.cross(a, [1.0, 0, 0])
        if np.linalg.norm(axis) < 1e-6:
            axis = np.cross(a, [0, 1.0, 0])
        axis /= np.linalg.norm(axis)
        return 2 * np.outer(axis, axis) - np.eye(3)
    K = np.array([[0, -v[2], v[1]], [v[2], 0, -v[0]], [-v[1], v[0], 0]])
    return np.eye(3) + K + K @ K / (1 + c)


def _orient_with_patch_along(target, patch, rng):
    """orientation R (rows) such that R . BASE[patch] = target, random spin about target"""
    R = _rot_to(BASE[patch], target)
    phi = rng.uniform(0, 2 * np.pi)
    t = target / np.linalg.norm(target)
    K = np.array([[0, -t[2], t[1]], [t[2], 0, -t[0]], [-t[1], t[0], 0]])
    S = np.eye(3) + np.sin(phi) * K + (1 - np.cos(phi)) * K @ K
    return S @ R


def _tilted(d, cos_target, rng):
    """unit vector at angle arccos(cos_target) from unit vector d"""
    perp = np.cross(d, rng.normal(size=3))
    perp /= np.linalg.norm(perp)
    s = np.sqrt(max(0.0, 1 - cos_target * cos_target))
    return cos_target * d + s * perp


def build(n_pairs=3000, delta=0.12, cosmax=0.92, seed=20240611):
    rng = np.random.default_rng(seed)
    rc2 = (1 + delta) ** 2
    offsets = np.array([0.0, 1e-15, -1e-15, 3e-13, -3e-13, 1e-9, -1e-9, 1e-7, -1e-7, 1e-6, -1e-6, 5e-6, -5e-6, 1e-5, -1e-5, 2e-5, -2e-5, 1e-4, -1e-4])
    spacing = 3.0
    side = int(np.ceil(n_pairs ** (1.0 / 3.0)))
    L = side * spacing
    r = np.zeros((2 * n_pairs, 3))
    R = np.zeros((2 * n_pairs, 9))
    for k in range(n_pairs):
        ix, iy, iz = k % side, (k // side) % side, k // (side * side)
        c = np.array([ix + 0.5, iy + 0.5, iz + 0.5]) * spacing
        kind = k % 4
        off = offsets[rng.integers(len(offsets))]
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        if kind == 0:  # contact distance
            r2 = 1.0 + off
        elif kind == 1:  # bond range edge
            r2 = rc2 + off
        else:  # inside the bond range, cosine near cosmax
            r2 = rng.uniform(1.0 + 1e-3, rc2 - 1e-3)
        dist = np.sqrt(r2)
        pa, qa = rng.integers(4), rng.integers(4)
        if kind == 2:  # p's cosine near threshold, q's comfortably above
            cp = cosmax + off
            cq = rng.uniform(cosmax + 0.01, 1.0)
        elif kind == 3:  # q's cosine near threshold
            cp = rng.uniform(cosmax + 0.01, 1.0)
            cq = cosmax + off
        else:
            cp = rng.uniform(cosmax - 0.05, 1.0)
            cq = rng.uniform(cosmax - 0.05, 1.0)
        Rp = _orient_with_patch_along(_tilted(d, min(cp, 1.0), rng), pa, rng)
        Rq = _orient_with_patch_along(_tilted(-d, min(cq, 1.0), rng), qa, rng)
        r[2 * k] = c - 0.5 * dist * d
        r[2 * k + 1] = c + 0.5 * dist * d
        R[2 * k] = Rp.reshape(9)
        R[2 * k + 1] = Rq.reshape(9)
    return r, R, np.array([L, L, L])


def write_rrr17(path, r, R, box):
    """.rrr layout (output.c:302-317) but with 17 significant digits everywhere"""
    with open(path, "w") as f:
        f.write("0 %d %.17g %.17g %.17g\n" % (len(r), box[0], box[1], box[2]))
        for i in range(len(r)):
            f.write("%.17g %.17g %.17g\n" % tuple(R[i, 0:3]))
            f.write("%.17g %.17g %.17g\n" % tuple(R[i, 3:6]))
            f.write("%.17g %.17g %.17g\n" % tuple(r[i]))
