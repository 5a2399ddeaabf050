"""The batched planner's exact early rejection (batch_kernel.cuh:
stage_domains, early_near, sample_group), restated in float32 numpy.

After 4 digit trips each coordinate is bounded by [h, h + w] with
w = f * b * (1 + 2^-10) + 2^-20 (nothing once the index is exhausted),
shifted by the scrambling rotation unless that wraps past 1, and mapped by
the monotone fmaf(v, scale, offset).  Checked here: (1) every finished
coordinate lies in its interval, for every base the samplers use, scrambled
or not; (2) no sample that the early test rejects (its interval box outside
every node's widened domain) passes the full dynamic-domain test (nearest
node's radius >= distance), on random trapped-tree node sets."""
import numpy as np

PRIMES = [3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59]
REL, ABS_R, ABS_H = np.float32(1 / 1024), np.float32(1 / 65536), np.float32(1 / 1048576)
f32 = np.float32


def fma32(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(np.float32)


def digits(it, b, a, trips=None):
    """Radical inverse of it (uint64 array) in base b with digits scrambled
    by a; stops after `trips` trips (None: to the end).  Returns (h, f, idx)."""
    it = it.copy()
    inv = f32(1.0) / f32(b)
    h = np.zeros(it.shape, np.float32)
    f = np.full(it.shape, inv, np.float32)
    k = 0
    while (it > 0).any() and (trips is None or k < trips):
        q = it // b
        dig = (a * (it - q * b)) % b
        h = fma32(f, dig.astype(np.float32), h)
        it = q
        f = (f * inv).astype(np.float32)
        k += 1
    return h, f, it


def interval(h, f, idx, b, rot, scale, offset, scramble):
    w = np.where(idx > 0, fma32(f * f32(b), np.full_like(f, f32(1) + REL), np.full_like(f, ABS_H)), f32(0))
    vlo, vhi = h.copy(), (h + w).astype(np.float32)
    if scramble:
        vlo, vhi = (vlo + rot).astype(np.float32), (vhi + rot).astype(np.float32)
        wrapped = vlo >= 1
        straddle = ~wrapped & (vhi >= 1)
        vlo = np.where(wrapped, vlo - f32(1), np.where(straddle, f32(0), vlo)).astype(np.float32)
        vhi = np.where(wrapped, vhi - f32(1), np.where(straddle, f32(1), vhi)).astype(np.float32)
    qa = fma32(vlo, np.full_like(vlo, scale), np.full_like(vlo, offset))
    qb = fma32(vhi, np.full_like(vhi, scale), np.full_like(vhi, offset))
    return np.minimum(qa, qb), np.maximum(qa, qb)


def final_coord(h, rot, scale, offset, scramble):
    if scramble:
        h = (h + rot).astype(np.float32)
        h = (h - np.floor(h)).astype(np.float32)
    return fma32(h, np.full_like(h, scale), np.full_like(h, offset))


def test_interval_contains_final_coordinate():
    rng = np.random.default_rng(0)
    it = np.concatenate([rng.integers(1, 1 << 31, 20000, dtype=np.uint64), np.arange(1, 2000, dtype=np.uint64)])
    for b in PRIMES:
        for scramble in (False, True):
            a = int(rng.integers(1, b)) if scramble else 1
            rot = f32(int(rng.integers(0, 1 << 24)) / 16777216.0) if scramble else f32(0)
            scale, offset = f32(rng.uniform(0.5, 6.0)), f32(rng.uniform(-3.0, 0.0))
            h4, f4, idx4 = digits(it, b, a, trips=4)
            lo, hi = interval(h4, f4, idx4, b, rot, scale, offset, scramble)
            q = final_coord(digits(it, b, a)[0], rot, scale, offset, scramble)
            assert (q >= lo).all() and (q <= hi).all(), (b, scramble)


def test_early_rejection_implies_full_rejection():
    rng = np.random.default_rng(1)
    D, n = 7, 30000
    bases = np.array(PRIMES[:D])
    scale = rng.uniform(3.0, 5.8, D).astype(np.float32)
    offset = (-scale / 2).astype(np.float32)
    it = rng.integers(1, 1 << 31, n, dtype=np.uint64)
    lo = np.empty((n, D), np.float32)
    hi = np.empty((n, D), np.float32)
    q = np.empty((n, D), np.float32)
    for d in range(D):
        a = int(rng.integers(1, bases[d]))
        rot = f32(int(rng.integers(0, 1 << 24)) / 16777216.0)
        h4, f4, idx4 = digits(it, int(bases[d]), a, trips=4)
        lo[:, d], hi[:, d] = interval(h4, f4, idx4, int(bases[d]), rot, scale[d], offset[d], True)
        q[:, d] = final_coord(digits(it, int(bases[d]), a)[0], rot, scale[d], offset[d], True)
    rejected_early = 0
    for trial in range(20):
        cnt = int(rng.integers(1, 33))
        centre = rng.uniform(offset, offset + scale).astype(np.float32)
        nodes = (centre + rng.normal(0, 0.3, (cnt, D))).astype(np.float32)
        radius = rng.choice([1.0, 1.3, 2.0, 4.0], cnt).astype(np.float32)
        # the kernel's early test
        m = fma32(radius, np.full(cnt, f32(1) + REL), np.full(cnt, ABS_R))
        rad2 = (m * m).astype(np.float32)
        box_lo = (nodes - m[:, None]).min(0)
        box_hi = (nodes + m[:, None]).max(0)
        in_box = ~((hi < box_lo) | (lo > box_hi)).any(1)
        gap = np.maximum(np.maximum(nodes[None] - hi[:, None], lo[:, None] - nodes[None]), f32(0))
        near = ((gap * gap).sum(2, dtype=np.float32) <= rad2[None]).any(1)
        early = ~(in_box & near) if cnt > 8 else ~near
        # the full test: nearest node by squared distance, accepted unless radius < distance
        d2 = ((q[:, None] - nodes[None]) ** 2).sum(2, dtype=np.float32)
        bi = d2.argmin(1)
        accepted = ~(radius[bi] < np.sqrt(d2[np.arange(n), bi]))
        assert not (early & accepted).any(), trial
        rejected_early += int(early.sum())
    assert rejected_early > 0.3 * 20 * n   # the test is selective, not vacuous
