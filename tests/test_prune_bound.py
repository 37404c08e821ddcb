"""The error lower bound behind the pipeline's pruning (qe_lower_bound in
fastc_gb300/csrc/bc7_intqe.cuh: the larger of a line term and a
palette-size term), restated step for step in float32 and
checked against the least error any BC7 palette of 4, 8 or 16 colours can
reach: for every texel the nearest palette colour, which is never worse
than the colour FasTC's QuantizedError picks. The endpoints are random and
fitted (the rounded extremes of the best line, where the bound is
tightest), on clusters from scattered to nearly collinear. A fit is only
pruned when its bound exceeds another candidate's error, so the bound
must never exceed an error that is reachable."""
import numpy as np

WEIGHTS = {
    2: [0, 21, 43, 64],
    3: [0, 9, 18, 27, 37, 46, 55, 64],
    4: [0, 4, 9, 13, 17, 21, 26, 30, 34, 38, 43, 47, 51, 55, 60, 64],
}


def level_term(px: np.ndarray, a: np.ndarray, levels: int) -> float:
    """The palette-size term of qe_lower_bound, in the kernel's steps."""
    n = px.shape[0]
    if levels != 4 or n <= levels:
        return 0.0
    d0 = int(np.argmax(np.diag(a)))  # first largest diagonal entry
    for c in range(4):
        if a[c, c] > a[d0, d0]:
            d0 = c
    u = a[:, d0].astype(np.float32).copy()
    for _ in range(4):
        w = np.zeros(4, np.float32)
        for r in range(4):
            w[r] = np.float32(np.float32(np.float32(a[r, 0] * u[0]) + np.float32(a[r, 1] * u[1]))
                              + np.float32(a[r, 2] * u[2])) + np.float32(a[r, 3] * u[3])
        mx = np.float32(np.abs(w).max())
        if not mx > 0:
            return 0.0
        u = (w * np.float32(np.float32(1.0) / mx)).astype(np.float32)
    um = np.float32(np.abs(u).max())
    d = np.rint((u * np.float32(64.0)) / um).astype(np.int64)
    dd = int((d * d).sum())
    if dd == 0:
        return 0.0
    sp = np.sort(px.astype(np.int64) @ d)
    g = np.sort(np.diff(sp))
    G = np.float32(int(g[:n - levels].sum()))
    return float(np.float32(np.float32(G * G) / np.float32(2 * levels * dd)) * np.float32(1.0 - 1e-5))


def lower_bound(px: np.ndarray, levels: int = 16) -> float:
    """qe_lower_bound for n texels (n x 4 bytes) and a `levels`-colour
    palette, in the kernel's steps."""
    n = px.shape[0]
    v = px.astype(np.int64)
    s = v.sum(0)
    q = v.T @ v
    m = n * q - np.outer(s, s)  # n * scatter, exact integers
    tr = int(np.trace(m))
    if tr <= 0:
        return 0.0
    a = m.astype(np.float32) * np.float32(1.0 / np.float32(tr))
    b = (a @ a).astype(np.float32)
    f = np.float32((b * b).sum())
    lam = np.float32(np.sqrt(np.sqrt(f)))
    r = np.float32(max(0.0, 1.0 - lam - 1e-5)) * np.float32(tr / n)
    r = float(r)
    line = max(0.0, r - 2.0 * np.sqrt(n * r) - 1e-3 * r) if r >= n else 0.0
    return max(line, level_term(px, a, levels))


def palette(q1: np.ndarray, q2: np.ndarray, bits: int) -> np.ndarray:
    w = np.array(WEIGHTS[bits], dtype=np.int64)[:, None]
    return (q1[None, :].astype(np.int64) * (64 - w) + q2[None, :].astype(np.int64) * w + 32) >> 6


def best_error(px: np.ndarray, pal: np.ndarray) -> int:
    d = px[:, None, :].astype(np.int64) - pal[None, :, :]
    return int((d * d).sum(2).min(1).sum())


def fitted_endpoints(px: np.ndarray, rng) -> tuple[np.ndarray, np.ndarray]:
    x = px.astype(np.float64)
    mean = x.mean(0)
    _, _, vt = np.linalg.svd(x - mean, full_matrices=False)
    t = (x - mean) @ vt[0]
    e1 = mean + vt[0] * t.min() + rng.normal(0, 1.0, 4)
    e2 = mean + vt[0] * t.max() + rng.normal(0, 1.0, 4)
    return (np.clip(np.rint(e1), 0, 255).astype(np.int64),
            np.clip(np.rint(e2), 0, 255).astype(np.int64))


def clusters(rng, count: int):
    for k in range(count):
        n = int(rng.integers(2, 17))
        kind = k % 4
        if kind == 0:  # scattered
            px = rng.integers(0, 256, (n, 4))
        elif kind == 1:  # near a line, small noise
            a, b = rng.integers(0, 256, 4), rng.integers(0, 256, 4)
            t = rng.random(n)[:, None]
            px = np.clip(np.rint(a + (b - a) * t + rng.normal(0, rng.choice([0.5, 2, 6]), (n, 4))), 0, 255)
        elif kind == 2:  # two blobs
            c = rng.integers(0, 256, (2, 4))
            px = np.clip(c[rng.integers(0, 2, n)] + rng.integers(-12, 13, (n, 4)), 0, 255)
        else:  # opaque, colour noise
            px = rng.integers(0, 256, (n, 4))
            px[:, 3] = 255
        yield px.astype(np.int64)


def test_bound_never_exceeds_a_reachable_error():
    rng = np.random.default_rng(20240611)
    checked = tight = 0
    for px in clusters(rng, 1200):
        for bits in (2, 3, 4):
            lb = lower_bound(px, 1 << bits)
            pairs = [fitted_endpoints(px, rng) for _ in range(3)]
            pairs += [(rng.integers(0, 256, 4), rng.integers(0, 256, 4)) for _ in range(2)]
            for q1, q2 in pairs:
                err = best_error(px, palette(q1, q2, bits))
                assert lb <= err, (px.tolist(), q1.tolist(), q2.tolist(), bits, lb, err)
                checked += 1
                tight += lb > 0.5 * err
    assert checked == 1200 * 3 * 5
    assert tight > 100  # the bound is not vacuous on these clusters


def test_palette_size_term_is_tight_on_a_uniform_ramp():
    """Sixteen texels evenly spread on a line: no 4-colour palette beats
    the best 4-level quantisation of the ramp (computed here by dynamic
    programming), and the palette-size term reaches 90 % of it (runs of
    four texels, 12 gaps: 12^2 / 8 = 18 squared steps against 4 x 5 =
    20)."""
    px = np.array([[16 * i, 8 * i, 255 - 4 * i, 255] for i in range(16)], dtype=np.int64)
    t = np.sort(px @ np.array([16, 8, -4, 0]) / np.sqrt(16 * 16 + 64 + 16))

    def opt(vals, k):  # exact 1-D k-means by dynamic programming
        n = len(vals)
        cost = lambda a, b: float(((vals[a:b] - vals[a:b].mean()) ** 2).sum()) if b > a else 0.0
        f = [cost(0, j) for j in range(n + 1)]
        for _ in range(k - 1):
            f = [min(f[a] + cost(a, j) for a in range(j + 1)) if j else 0.0 for j in range(n + 1)]
        return f[n]

    lb = lower_bound(px, 4)
    best = opt(t, 4)
    assert 0.85 * best <= lb <= best + 1e-6, (lb, best)


def test_bound_is_zero_for_collinear_and_tiny_clusters():
    px = np.array([[10 * i, 5 * i, 255 - 3 * i, 255] for i in range(16)], dtype=np.int64)
    assert lower_bound(px) == 0.0
    assert lower_bound(np.array([[1, 2, 3, 4], [200, 100, 50, 25]], dtype=np.int64)) == 0.0
    assert lower_bound(np.full((16, 4), 77, dtype=np.int64)) == 0.0
