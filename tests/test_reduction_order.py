"""The summation orders the kernels rely on, restated on the host (no GPU).

The power-step loop's reduction warp (warp_item_sums in engine.cu) sums an
instance's item partials in rounds of kSumStage staged items, lane l keeping
the running sums of finalize threads l, l+32, ..., l+224.  Its result must be
bitwise the launch form's finalize: thread t sums items t, t+256, ... in
order, block_reduce's warp adds the threads' sums l, l+32, ..., l+224, and a
shuffle tree closes.  The GPU tests check the two kernels against each other
for instances of up to 1,536 items (one round); this restatement checks the
orders agree for any item count, including several rounds.

The cluster solver's cross-CTA reduction for clusters of up to 32 items runs
as one warp per slot: lane l takes item l and then adds the seven identity
terms the block reduction would add from threads that hold no item, so even
a -0.0 partial comes out as the block reduction leaves it."""
import numpy as np
import pytest

K_THREADS = 256
K_SUM_STAGE = 6 * K_THREADS


def warp_sum(v):
    """__shfl_xor_sync butterfly: every lane adds its partner at 16, 8, 4, 2, 1."""
    v = v.copy()
    for o in (16, 8, 4, 2, 1):
        v = v + v[np.arange(32) ^ o]
    return v[0]


def finalize_order(p):
    """phase_item's finalize followed by block_reduce (two slots)."""
    acc = np.zeros((K_THREADS, 2))
    for t in range(K_THREADS):
        for it in range(t, len(p), K_THREADS):
            acc[t] += p[it]
    out = []
    for k in range(2):
        a = acc[0:32, k].copy()
        for i in range(1, K_THREADS // 32):
            a = a + acc[32 * i:32 * i + 32, k]
        out.append(warp_sum(a))
    return out


def staged_warp_order(p):
    """warp_item_sums: staged rounds, then per round the sixteen sums of lane l."""
    t = np.zeros((32, K_THREADS // 32, 2))
    for base in range(0, len(p), K_SUM_STAGE):
        stage = p[base:base + K_SUM_STAGE]
        n = len(stage)
        for r in range(0, n, K_THREADS):
            for lane in range(32):
                for i in range(K_THREADS // 32):
                    j = r + lane + 32 * i
                    if j < n:
                        t[lane, i] += stage[j]
    out = []
    for k in range(2):
        a = t[:, 0, k].copy()
        for i in range(1, K_THREADS // 32):
            a = a + t[:, i, k]
        out.append(warp_sum(a))
    return out


def _partials(nitems):
    # signed values over six decades: any change of the order changes the bits
    rng = np.random.default_rng(nitems)
    return rng.standard_normal((nitems, 2)) * 10.0 ** rng.uniform(-3, 3, size=(nitems, 1))


@pytest.mark.parametrize("nitems", [1, 37, 256, 549, 1360, 1536, 1537, 1601, 3072, 4000])
def test_staged_warp_sums_follow_the_finalize_order(nitems):
    p = _partials(nitems)
    got, want = staged_warp_order(p), finalize_order(p)
    assert got[0] == want[0] and got[1] == want[1]


def test_the_check_sees_a_changed_order():
    """Reversing the rounds inside a stage (same items, other order) is caught."""
    p = _partials(4000)
    t = np.zeros((32, K_THREADS // 32, 2))
    for base in range(0, len(p), K_SUM_STAGE):
        stage = p[base:base + K_SUM_STAGE]
        for r in reversed(range(0, len(stage), K_THREADS)):
            for lane in range(32):
                for i in range(K_THREADS // 32):
                    j = r + lane + 32 * i
                    if j < len(stage):
                        t[lane, i] += stage[j]
    a = t[:, 0, 0].copy()
    for i in range(1, K_THREADS // 32):
        a = a + t[:, i, 0]
    assert warp_sum(a) != finalize_order(p)[0]


def block_reduce_of_items(vals, is_min=False):
    """The cluster solver's general cross-CTA path for one slot: thread t
    takes item t (identity start), then block_reduce's warp, then the tree."""
    ident = np.finfo(np.float64).max if is_min else 0.0
    acc = np.full(K_THREADS, ident)
    for t, x in enumerate(vals):
        acc[t] = min(acc[t], x) if is_min else acc[t] + x
    a = acc[0:32].copy()
    for i in range(1, K_THREADS // 32):
        b = acc[32 * i:32 * i + 32]
        a = np.minimum(a, b) if is_min else a + b
    if is_min:
        v = a.copy()
        for o in (16, 8, 4, 2, 1):
            v = np.minimum(v, v[np.arange(32) ^ o])
        return v[0]
    return warp_sum(a)


def one_warp_of_items(vals, is_min=False):
    """The one-warp path (clusters of up to 32 items): lane l takes item l,
    then seven identity terms, then the tree."""
    ident = np.finfo(np.float64).max if is_min else 0.0
    a = np.full(32, ident)
    for l, x in enumerate(vals):
        a[l] = min(a[l], x) if is_min else a[l] + x
    for _ in range(1, K_THREADS // 32):
        a = np.minimum(a, ident) if is_min else a + 0.0
    if is_min:
        v = a.copy()
        for o in (16, 8, 4, 2, 1):
            v = np.minimum(v, v[np.arange(32) ^ o])
        return v[0]
    return warp_sum(a)


@pytest.mark.parametrize("nitems", [1, 2, 7, 16, 31, 32])
@pytest.mark.parametrize("is_min", [False, True])
def test_one_warp_cross_cta_reduction_is_the_block_reduction(nitems, is_min):
    vals = list(_partials(nitems)[:, 0])
    if nitems > 1:
        vals[1] = -0.0  # the identity terms keep what the block reduction does with it
    got, want = one_warp_of_items(vals, is_min), block_reduce_of_items(vals, is_min)
    assert np.float64(got).tobytes() == np.float64(want).tobytes()


def warp_finalize_of_items(vals, is_min=False):
    """warp_finalize (the engine's and the phase kernel's finalize for up to
    256 items): lane l forms, for i = 0..7, the value thread l + 32 i holds
    in the block form (the identity, plus item l + 32 i when there is one)
    and adds them in that order, then the tree."""
    ident = np.finfo(np.float64).max if is_min else 0.0
    a = np.zeros(32)
    for lane in range(32):
        acc = None
        for i in range(K_THREADS // 32):
            t = lane + 32 * i
            th = ident
            if t < len(vals):
                th = min(th, vals[t]) if is_min else th + vals[t]
            acc = th if i == 0 else (min(acc, th) if is_min else acc + th)
        a[lane] = acc
    if is_min:
        v = a.copy()
        for o in (16, 8, 4, 2, 1):
            v = np.minimum(v, v[np.arange(32) ^ o])
        return v[0]
    return warp_sum(a)


@pytest.mark.parametrize("nitems", [1, 17, 32, 33, 100, 255, 256])
@pytest.mark.parametrize("is_min", [False, True])
def test_warp_finalize_is_the_block_finalize(nitems, is_min):
    vals = list(_partials(nitems)[:, 0])
    if nitems > 40:
        vals[40] = -0.0
    got, want = warp_finalize_of_items(vals, is_min), block_reduce_of_items(vals, is_min)
    assert np.float64(got).tobytes() == np.float64(want).tobytes()
