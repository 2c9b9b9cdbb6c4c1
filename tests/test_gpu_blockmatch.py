"""GPU block matching through the C ABI vs the reference's known answers and the oracle."""

import ctypes
import zlib

import numpy as np
import pytest

from parity import compare_match_sets

pytestmark = pytest.mark.gpu


def _mp(counts, radius, max_m, min_m, code, stabilize=True, scale=1.0, pow2=True):
    from bmnd_gb300 import _abi

    p = _abi.MatchParams()
    p.ndim = len(counts)
    for a, (c, r) in enumerate(zip(counts, radius)):
        p.counts[a] = c
        p.search_radius[a] = r
    p.max_matches, p.min_matches = max_m, min_m
    p.prefer_power_of_two = int(pow2)
    p.distance = code
    p.stabilize_ties = int(stabilize)
    p.count_scale = scale
    return p


def gpu_match_patches(torch, native, patches, counts, refs, radius, max_m, min_m, thr, code,
                      stabilize=True, scale=1.0, pow2=True):
    from bmnd_gb300 import _abi

    dev = torch.device("cuda:0")
    pt = torch.from_numpy(np.ascontiguousarray(patches, dtype=np.float32)).to(dev)
    rt = torch.from_numpy(np.ascontiguousarray(refs, dtype=np.int32).reshape(-1, len(counts))).to(dev)
    n = rt.shape[0]
    tt = torch.full((max(n, 1),), float(np.float32(thr)), dtype=torch.float32, device=dev)
    sel = torch.full((max(n, 1), max_m), -7, dtype=torch.int32, device=dev)
    cnt = torch.zeros(max(n, 1), dtype=torch.int32, device=dev)
    acc = torch.zeros(max(n, 1), dtype=torch.int32, device=dev)
    p = _mp(counts, radius, max_m, min_m, code, stabilize, scale, pow2)
    _abi.check(native.bmnd_blockmatch_patches(ctypes.byref(p), pt.data_ptr(), pt.shape[1], rt.data_ptr(),
                                              n, tt.data_ptr(), sel.data_ptr(), cnt.data_ptr(),
                                              acc.data_ptr(), 0))
    torch.cuda.synchronize()
    return sel.cpu().numpy()[:n], cnt.cpu().numpy()[:n], acc.cpu().numpy()[:n]


def selected(sel, cnt, i):
    return sel[i, : cnt[i]].tolist()


SSD, DEV, PEARSON, ANSCOMBE = 0, 1, 2, 3


def _volume_match(torch, native, volume, block, refs, radius, max_m, min_m, thr, gamma=None, scale=1.0):
    """SSD matching over a volume through the C ABI; with ``gamma`` the Poisson
    SSD noise-bias correction (bmnd_blockmatch_volume_poisson_biased)."""
    from bmnd_gb300 import _abi

    dev = torch.device("cuda:0")
    vol = np.ascontiguousarray(volume, dtype=np.float32)
    counts = tuple(s - b + 1 for s, b in zip(vol.shape, block))
    vt = torch.from_numpy(vol).to(dev)
    rt = torch.from_numpy(np.ascontiguousarray(refs, dtype=np.int32).reshape(-1, vol.ndim)).to(dev)
    n = rt.shape[0]
    tt = torch.full((n,), float(np.float32(thr)), dtype=torch.float32, device=dev)
    sel = torch.full((n, max_m), -7, dtype=torch.int32, device=dev)
    cnt = torch.zeros(n, dtype=torch.int32, device=dev)
    acc = torch.zeros(n, dtype=torch.int32, device=dev)
    p = _mp(counts, radius, max_m, min_m, SSD, stabilize=False, scale=scale, pow2=False)
    shape = (ctypes.c_int32 * vol.ndim)(*vol.shape)
    blk = (ctypes.c_int32 * vol.ndim)(*block)
    if gamma is None:
        rc = native.bmnd_blockmatch_volume(ctypes.byref(p), vt.data_ptr(), shape, blk, rt.data_ptr(), n,
                                           tt.data_ptr(), sel.data_ptr(), cnt.data_ptr(), acc.data_ptr(), 0)
    else:
        rc = native.bmnd_blockmatch_volume_poisson_biased(ctypes.byref(p), vt.data_ptr(), shape, blk,
                                                          rt.data_ptr(), n, tt.data_ptr(), float(gamma),
                                                          sel.data_ptr(), cnt.data_ptr(), acc.data_ptr(), 0)
    _abi.check(rc)
    torch.cuda.synchronize()
    return sel.cpu().numpy(), cnt.cpu().numpy(), acc.cpu().numpy()


def test_poisson_gamma_corrects_ssd_noise_bias(cuda, native):
    # tests/test_blockmatching_internal_unit.py:203-229: patches [0] and [2],
    # threshold 1; the bias 1 * (0 + 2) times gamma 2 brings the SSD 4 to 0
    from bmnd_gb300 import _abi

    vol = np.array([0.0, 2.0], dtype=np.float32)
    sel, cnt, _ = _volume_match(cuda, native, vol, (1,), [[0]], (1,), 2, 1, 1.0)
    assert selected(sel, cnt, 0) == [0]
    n0 = _abi.launch_count()
    sel, cnt, acc = _volume_match(cuda, native, vol, (1,), [[0]], (1,), 2, 1, 1.0, gamma=2.0)
    assert _abi.launch_count() - n0 == 1  # one exact warp-kernel launch, counted by the library
    assert selected(sel, cnt, 0) == [0, 1]
    assert acc[0] == 2


def test_poisson_gamma_bias_order_and_centre(cuda, native):
    """Against a float32 restatement of the reference's loop (blockmatching.py:
    323-336, :432-443, :1114-1145) on a random 2-D volume with a count scale:
    accepted counts and match sets equal, the reference patch uncorrected."""
    rng = np.random.default_rng(5)
    vol = rng.poisson(6.0, size=(14, 13)).astype(np.float32)
    vol[3:6, 4:9] = 0.0
    block, radius, scale, gamma, thr, max_m = (4, 4), (3, 3), 0.75, 1.5, 40.0, 8
    counts = (vol.shape[0] - 3, vol.shape[1] - 3)
    refs = [(r, c) for r in range(0, counts[0], 2) for c in range(0, counts[1], 3)]
    sel, cnt, acc = _volume_match(cuda, native, vol, block, refs, radius, max_m, 1, thr, gamma=gamma, scale=scale)
    s32, g32 = np.float32(scale), np.float32(gamma)
    for i, (r0, c0) in enumerate(refs):
        ref = vol[r0:r0 + 4, c0:c0 + 4].reshape(-1)
        scored = []
        for r in range(max(r0 - 3, 0), min(r0 + 3, counts[0] - 1) + 1):
            for c in range(max(c0 - 3, 0), min(c0 + 3, counts[1] - 1) + 1):
                cand = vol[r:r + 4, c:c + 4].reshape(-1)
                d = np.float32(0.0)
                b = np.float32(0.0)
                for p in range(16):
                    diff = np.float32(cand[p] - ref[p])
                    d = np.float32(d + np.float32(diff * diff))
                    pooled = np.float32(ref[p] + cand[p])
                    if pooled > 0.0:
                        b = np.float32(b + np.float32(s32 * pooled))
                if (r, c) != (r0, c0):
                    d = np.float32(d - np.float32(g32 * b))
                scored.append((d, r * counts[1] + c))
        accepted = sorted(x for x in scored if x[0] < np.float32(thr))
        centre = r0 * counts[1] + c0
        # the row: the reference patch first, then the accepted by (distance, index)
        want = [centre] + [lin for _, lin in accepted if lin != centre][: max_m - 1]
        assert acc[i] == len(accepted), (i, acc[i], len(accepted))
        assert selected(sel, cnt, i) == want, (i, selected(sel, cnt, i), want)


def test_self_only_with_zero_radius(cuda, native):
    # tests/test_blockmatching_unit.py:11-30
    patches = np.array([[0.0, 0.0], [1.0, 1.0], [2.0, 2.0]], dtype=np.float32)
    sel, cnt, _ = gpu_match_patches(cuda, native, patches, (3,), [[0], [1], [2]], (0,), 2, 1, 1.0, SSD,
                                    stabilize=False, pow2=False)
    assert [selected(sel, cnt, i) for i in range(3)] == [[0], [1], [2]]


def test_includes_self_in_neighbors(cuda, native):
    # tests/test_blockmatching_unit.py:32-48
    patches = np.array([[0.0, 0.0], [1.0, 1.0], [2.0, 2.0]], dtype=np.float32)
    sel, cnt, _ = gpu_match_patches(cuda, native, patches, (3,), [[1]], (1,), 2, 1, 100.0, SSD,
                                    stabilize=False, pow2=False)
    assert selected(sel, cnt, 0) == [1, 0]


@pytest.mark.parametrize("code", [DEV, PEARSON, ANSCOMBE])
def test_poisson_distances_account_for_count_dependent_variance(cuda, native, code):
    # tests/test_blockmatching_unit.py:101-133
    patches = np.array([[0.0, 2.0], [2.0, 2.0], [1.0, 1.0]], dtype=np.float32)
    sel, cnt, _ = gpu_match_patches(cuda, native, patches, (3,), [[2]], (2,), 3, 1, 100.0, SSD,
                                    stabilize=False, pow2=False)
    assert selected(sel, cnt, 0) == [2, 0, 1]
    sel, cnt, _ = gpu_match_patches(cuda, native, patches, (3,), [[2]], (2,), 3, 1, 100.0, code,
                                    stabilize=False, pow2=False)
    assert selected(sel, cnt, 0) == [2, 1, 0]


@pytest.mark.parametrize("code", [DEV, PEARSON, ANSCOMBE])
def test_poisson_distances_are_invariant_to_representation_scale(cuda, native, code):
    # tests/test_blockmatching_unit.py:145-181
    counts_p = np.array([[11.0, 9.0], [10.0, 10.0], [20.0, 20.0]], dtype=np.float32)
    a, ca, _ = gpu_match_patches(cuda, native, counts_p, (3,), [[1]], (1,), 3, 1, 0.2, code,
                                 stabilize=False, pow2=False, scale=1.0)
    b, cb, _ = gpu_match_patches(cuda, native, 7.0 * counts_p, (3,), [[1]], (1,), 3, 1, 0.2, code,
                                 stabilize=False, pow2=False, scale=7.0)
    assert selected(a, ca, 0) == [1, 0]
    assert selected(b, cb, 0) == selected(a, ca, 0)


def test_min_stack_fill_from_rejected(cuda, native):
    # tests/test_blockmatching_internal_unit.py:96-109
    patches = np.array([[0.0], [10.0], [20.0], [30.0]], dtype=np.float32)
    sel, cnt, acc = gpu_match_patches(cuda, native, patches, (4,), [[1]], (3,), 4, 3, 1e-8, SSD,
                                      stabilize=False, pow2=False)
    assert acc[0] == 1 and cnt[0] == 3
    assert selected(sel, cnt, 0) == [1, 0, 2]


def test_tie_break_by_linear_index_and_reference_first(cuda, native):
    # ties at equal distance resolve by linear index; the reference leads
    patches = np.array([[5.0], [5.0], [5.0], [5.0], [5.0]], dtype=np.float32)
    sel, cnt, acc = gpu_match_patches(cuda, native, patches, (5,), [[3]], (4,), 4, 1, 1.0, DEV,
                                      stabilize=True, pow2=False)
    assert selected(sel, cnt, 0) == [3, 0, 1, 2]
    assert acc[0] == 5


def test_power_of_two_truncation(cuda, native):
    patches = np.arange(7, dtype=np.float32).reshape(7, 1)
    sel, cnt, _ = gpu_match_patches(cuda, native, patches, (7,), [[3]], (3,), 16, 2, 100.0, SSD,
                                    stabilize=False, pow2=True)
    assert cnt[0] == 4
    assert selected(sel, cnt, 0) == [3, 2, 4, 1]


def test_batch_and_order_invariance(cuda, native):
    rng = np.random.default_rng(3)
    patches = rng.poisson(8.0, size=(50, 9)).astype(np.float32)
    refs = np.arange(50).reshape(-1, 1)
    a = gpu_match_patches(cuda, native, patches, (50,), refs, (6,), 8, 2, 3.0, DEV)
    b = gpu_match_patches(cuda, native, patches, (50,), refs[::-1], (6,), 8, 2, 3.0, DEV)
    np.testing.assert_array_equal(a[0], b[0][::-1])
    np.testing.assert_array_equal(a[1], b[1][::-1])


@pytest.mark.parametrize("code", [SSD, DEV, PEARSON, ANSCOMBE])
def test_patch_table_matches_oracle_2d(cuda, native, oracle_lib, code):
    rng = np.random.default_rng(100 + code)
    counts = (23, 31)
    lam = rng.uniform(0.5, 30.0, size=(counts[0] * counts[1], 1))
    patches = rng.poisson(lam, size=(counts[0] * counts[1], 16)).astype(np.float32)
    refs = np.array([(i, j) for i in range(0, counts[0], 2) for j in range(0, counts[1], 3)], dtype=np.int32)
    thr = 1e9 if code == SSD else 2.5
    g = gpu_match_patches(cuda, native, patches, counts, refs, (5, 4), 16, 2, thr, code,
                          stabilize=code != SSD)
    o = oracle_lib.blockmatch_patches(patches, counts, refs, (5, 4), 16, 2, thr, code,
                                      stabilize=code != SSD)
    np.testing.assert_array_equal(g[2], o[2])
    np.testing.assert_array_equal(g[1], o[1])
    assert np.mean(np.all(g[0] == o[0], axis=1)) >= 0.98


@pytest.mark.parametrize("shape,block,radius,max_m,thr", [
    ((48, 40), (8, 8), (19, 19), 16, 2.9527),
    ((48, 40), (8, 8), (19, 19), 32, 0.3937),
    ((20, 22, 18), (4, 4, 4), (7, 7, 7), 16, 2.9527),
    ((20, 22, 18), (5, 5, 5), (7, 7, 7), 32, 0.7689),
])
def test_volume_matching_vs_oracle(cuda, native, oracle_lib, shape, block, radius, max_m, thr):
    from bmnd_gb300 import _abi

    rng = np.random.default_rng(sum(shape))
    base = rng.uniform(1.0, 40.0, size=shape)
    vol = rng.poisson(base).astype(np.float32)
    counts = tuple(s - b + 1 for s, b in zip(shape, block))
    refs = np.stack(np.meshgrid(*[np.arange(0, c, 3) for c in counts], indexing="ij"), -1).reshape(-1, len(shape))
    refs = refs.astype(np.int32)
    dev = cuda.device("cuda:0")
    vt = cuda.from_numpy(vol).to(dev)
    rt = cuda.from_numpy(refs).to(dev)
    n = refs.shape[0]
    tt = cuda.full((n,), float(np.float32(thr)), device=dev)
    sel = cuda.empty((n, max_m), dtype=cuda.int32, device=dev)
    cnt = cuda.empty(n, dtype=cuda.int32, device=dev)
    acc = cuda.empty(n, dtype=cuda.int32, device=dev)
    p = _mp(counts, radius, max_m, 2, DEV)
    sh = (ctypes.c_int32 * len(shape))(*shape)
    bl = (ctypes.c_int32 * len(shape))(*block)
    _abi.check(native.bmnd_blockmatch_volume(ctypes.byref(p), vt.data_ptr(), sh, bl, rt.data_ptr(), n,
                                             tt.data_ptr(), sel.data_ptr(), cnt.data_ptr(), acc.data_ptr(), 0))
    cuda.cuda.synchronize()
    gs, gc, ga = sel.cpu().numpy(), cnt.cpu().numpy(), acc.cpu().numpy()
    os_, oc, oa = oracle_lib.blockmatch_volume(vol, block, refs, radius, max_m, 2, thr, DEV)
    eq, tied, bad = compare_match_sets(oracle_lib, vol, block, refs, gs, gc, os_, oc, DEV, thr)
    assert not bad, f"unexplained match-set differences in rows {bad[:10]}"
    assert eq >= 0.98 * n
    assert np.mean(ga == oa) >= 0.98


def _match_volume(cuda, native, vol, block, radius, max_m, min_m, thr, precision, refs=None):
    from bmnd_gb300 import _abi

    shape = vol.shape
    counts = tuple(s - b + 1 for s, b in zip(shape, block))
    if refs is None:
        refs = np.stack(np.meshgrid(*[np.arange(0, c, 2) for c in counts], indexing="ij"), -1)
        refs = refs.reshape(-1, len(shape)).astype(np.int32)
    dev = cuda.device("cuda:0")
    vt = cuda.from_numpy(np.ascontiguousarray(vol, dtype=np.float32)).to(dev)
    rt = cuda.from_numpy(refs).to(dev)
    n = refs.shape[0]
    tt = cuda.full((n,), float(np.float32(thr)), device=dev)
    sel = cuda.full((n, max_m), -7, dtype=cuda.int32, device=dev)
    cnt = cuda.full((n,), -7, dtype=cuda.int32, device=dev)
    acc = cuda.full((n,), -7, dtype=cuda.int32, device=dev)
    p = _mp(counts, radius, max_m, min_m, DEV)
    p.precision = precision
    sh = (ctypes.c_int32 * len(shape))(*shape)
    bl = (ctypes.c_int32 * len(shape))(*block)
    _abi.check(native.bmnd_blockmatch_volume(ctypes.byref(p), vt.data_ptr(), sh, bl, rt.data_ptr(), n,
                                             tt.data_ptr(), sel.data_ptr(), cnt.data_ptr(), acc.data_ptr(), 0))
    cuda.cuda.synchronize()
    return sel.cpu().numpy(), cnt.cpu().numpy(), acc.cpu().numpy()


@pytest.mark.parametrize("shape,block,radius,max_m,thr", [
    ((40, 44), (8, 8), (19, 19), 32, 0.3937),
    ((40, 44), (8, 8), (19, 19), 16, 2.9527),
    ((22, 20, 24), (5, 5, 5), (7, 7, 7), 32, 0.7689),
    ((22, 20, 24), (4, 4, 4), (7, 7, 7), 16, 2.9527),
])
@pytest.mark.parametrize("kind", ["smooth", "tiny", "sparse", "large", "flat"])
def test_screened_matching_equals_exact(cuda, native, shape, block, radius, max_m, thr, kind):
    """The screened deviance path (precision=fast) must give bit-identical match tables."""
    from bmnd_gb300 import _abi

    rng = np.random.default_rng(hash((shape, kind)) % 2**32)
    grids = np.meshgrid(*[np.linspace(0, 1, s) for s in shape], indexing="ij")
    smooth = 5.0 + 20.0 * np.sin(3 * grids[0]) ** 2 + 10.0 * grids[-1]
    if kind == "smooth":
        vol = smooth + rng.normal(0, 0.5, size=shape)
    elif kind == "tiny":
        vol = rng.uniform(0.0, 0.05, size=shape)
    elif kind == "sparse":
        vol = rng.poisson(0.3, size=shape) * rng.uniform(0.5, 1.5, size=shape)
    elif kind == "large":
        vol = 500.0 * smooth + rng.normal(0, 30.0, size=shape)
    else:
        vol = np.full(shape, 7.25) + (rng.random(shape) < 0.02) * 3.0
    vol = np.maximum(vol, 0.0).astype(np.float32)
    ex = _match_volume(cuda, native, vol, block, radius, max_m, 2, thr, _abi.MATCH_EXACT)
    fa = _match_volume(cuda, native, vol, block, radius, max_m, 2, thr, _abi.MATCH_FAST)
    np.testing.assert_array_equal(fa[1], ex[1])
    np.testing.assert_array_equal(fa[2], ex[2])
    np.testing.assert_array_equal(fa[0], ex[0])


def test_screened_fallback_when_threshold_rejects_everything(cuda, native):
    """Only the reference is accepted: the best rejected fill comes from the exact redo."""
    from bmnd_gb300 import _abi

    rng = np.random.default_rng(5)
    vol = rng.uniform(1.0, 50.0, size=(30, 30)).astype(np.float32)
    ex = _match_volume(cuda, native, vol, (8, 8), (5, 5), 16, 2, 1e-7, _abi.MATCH_EXACT)
    fa = _match_volume(cuda, native, vol, (8, 8), (5, 5), 16, 2, 1e-7, _abi.MATCH_FAST)
    assert np.all(ex[1] == 2)
    for i in range(3):
        np.testing.assert_array_equal(fa[i], ex[i])


def _exact_deviance(vol, block, counts, ref_lin, cand_lin):
    """Mean Poisson-deviance term (float64) between the patches at two patch-grid linear indices."""
    ra = np.array(np.unravel_index(ref_lin, counts))
    ca = np.array(np.unravel_index(np.asarray(cand_lin), counts))
    r = vol[tuple(slice(int(o), int(o) + b) for o, b in zip(ra, block))].astype(np.float64).ravel()
    out = []
    for k in range(ca.shape[1]):
        c = vol[tuple(slice(int(o), int(o) + b) for o, b in zip(ca[:, k], block))].astype(np.float64).ravel()
        s = r + c
        with np.errstate(divide="ignore", invalid="ignore"):
            t = np.where(r > 0, r * np.log(2 * r / s), 0.0) + np.where(c > 0, c * np.log(2 * c / s), 0.0)
        out.append(2.0 * t.sum() / r.size)
    return np.array(out)


@pytest.mark.parametrize("shape,block,radius,max_m,thr", [
    ((22, 20, 24), (5, 5, 5), (7, 7, 7), 16, 2.9527),
    ((21, 23, 19), (4, 4, 4), (6, 7, 5), 16, 2.9527),
    ((46, 41), (8, 8), (19, 19), 16, 2.9527),
])
@pytest.mark.parametrize("kind", ["smooth", "counts"])
def test_approx_matching_selects_near_optimal_groups(cuda, native, shape, block, radius, max_m, thr, kind):
    """precision=approx ranks candidates by the box-sum screening form without
    a bound.  Its groups must match the exact groups in size for almost every
    reference, and their summed exact distances may exceed the exact optimum
    only by rounding-level amounts."""
    from bmnd_gb300 import _abi

    rng = np.random.default_rng(17 + len(shape))
    grids = np.meshgrid(*[np.linspace(0, 1, s) for s in shape], indexing="ij")
    smooth = 5.0 + 20.0 * np.sin(3 * grids[0]) ** 2 + 10.0 * grids[-1]
    if kind == "smooth":
        vol = smooth + rng.normal(0, 0.5, size=shape)
    else:
        vol = rng.poisson(smooth).astype(np.float64)
    vol = np.maximum(vol, 0.0).astype(np.float32)
    counts = tuple(s - b + 1 for s, b in zip(shape, block))
    refs = np.stack(np.meshgrid(*[np.arange(0, c, 3) for c in counts], indexing="ij"), -1)
    refs = refs.reshape(-1, len(shape)).astype(np.int32)
    ex = _match_volume(cuda, native, vol, block, radius, max_m, 2, thr, _abi.MATCH_EXACT, refs)
    ap = _match_volume(cuda, native, vol, block, radius, max_m, 2, thr, _abi.MATCH_APPROX, refs)
    same = ap[1] == ex[1]
    assert same.mean() >= 0.97, same.mean()
    worse, tot_a, tot_e = 0, 0.0, 0.0
    for i in np.flatnonzero(same):
        rl = int(np.ravel_multi_index(tuple(refs[i]), counts))
        assert ap[0][i, 0] == rl  # the reference leads its group
        da = _exact_deviance(vol, block, counts, rl, ap[0][i, : ap[1][i]]).sum()
        de = _exact_deviance(vol, block, counts, rl, ex[0][i, : ex[1][i]]).sum()
        tot_a += da
        tot_e += de
        if da > de * (1 + 1e-3) + 1e-6:
            worse += 1
    assert worse <= 0.02 * same.sum(), (worse, same.sum())
    assert tot_a <= tot_e * (1 + 1e-4) + 1e-6, (tot_a, tot_e)


@pytest.mark.parametrize("shape,block,radius,max_m,thr", [
    ((22, 20, 24), (5, 5, 5), (7, 7, 7), 16, 2.9527),
    ((46, 41), (8, 8), (19, 19), 16, 2.9527),
])
def test_subsampled_matching_selects_good_groups(cuda, native, shape, block, radius, max_m, thr):
    """precision=subsampled prescreens on the patch's even sub-lattice, so its
    groups may differ from the exact ones more often than approx's; their
    summed exact distances must stay within 2% of the exact optimum overall."""
    from bmnd_gb300 import _abi

    rng = np.random.default_rng(41 + len(shape))
    grids = np.meshgrid(*[np.linspace(0, 1, s) for s in shape], indexing="ij")
    smooth = 5.0 + 20.0 * np.sin(3 * grids[0]) ** 2 + 10.0 * grids[-1]
    vol = np.maximum(smooth + rng.normal(0, 0.5, size=shape), 0.0).astype(np.float32)
    counts = tuple(s - b + 1 for s, b in zip(shape, block))
    refs = np.stack(np.meshgrid(*[np.arange(0, c, 3) for c in counts], indexing="ij"), -1)
    refs = refs.reshape(-1, len(shape)).astype(np.int32)
    ex = _match_volume(cuda, native, vol, block, radius, max_m, 2, thr, _abi.MATCH_EXACT, refs)
    sb = _match_volume(cuda, native, vol, block, radius, max_m, 2, thr, _abi.MATCH_SUBSAMPLED, refs)
    same = sb[1] == ex[1]
    assert same.mean() >= 0.95, same.mean()
    tot_s = tot_e = 0.0
    for i in np.flatnonzero(same):
        rl = int(np.ravel_multi_index(tuple(refs[i]), counts))
        assert sb[0][i, 0] == rl
        tot_s += _exact_deviance(vol, block, counts, rl, sb[0][i, : sb[1][i]]).sum()
        tot_e += _exact_deviance(vol, block, counts, rl, ex[0][i, : ex[1][i]]).sum()
    assert tot_s <= tot_e * 1.02 + 1e-6, (tot_s, tot_e)


def _patch_table(vol, block):
    """patches_flat of a volume: row = patch-grid linear index, column = patch element (C order)."""
    win = np.lib.stride_tricks.sliding_window_view(vol, block)
    counts = win.shape[: vol.ndim]
    return np.ascontiguousarray(win.reshape(int(np.prod(counts)), int(np.prod(block)))), counts


@pytest.mark.parametrize("shape,block,radius,max_m,thr", [
    ((40, 44), (8, 8), (19, 19), 16, 2.9527),
    ((22, 20, 24), (4, 4, 4), (7, 7, 7), 16, 2.9527),
    ((20, 22, 18), (5, 5, 5), (7, 7, 7), 32, 0.7689),
    ((18, 21, 16), (3, 4, 2), (5, 4, 6), 16, 2.9527),
])
@pytest.mark.parametrize("kind", ["counts", "mixed", "bright"])
def test_count_tabulated_volume_matching_equals_patch_table(cuda, native, shape, block, radius, max_m, thr,
                                                              kind):
    """The integer-count tabulated volume kernel and the per-term patch-table
    kernel are independent implementations of the same exact distance: their
    match tables must be bit-identical, also where voxels fall outside the
    table (non-integer, negative, or counts >= 63) and the reference patch is
    itself non-integer."""
    from bmnd_gb300 import _abi

    rng = np.random.default_rng(hash((shape, kind)) % 2**32)
    lam = {"counts": 20.0, "mixed": 20.0, "bright": 70.0}[kind]
    base = rng.uniform(0.2 * lam, 1.5 * lam, size=shape)
    vol = rng.poisson(base).astype(np.float32)
    if kind == "mixed":
        vol[rng.random(shape) < 0.03] += np.float32(0.25)
        vol[rng.random(shape) < 0.01] = np.float32(-1.0)
    counts = tuple(s - b + 1 for s, b in zip(shape, block))
    refs = np.stack(np.meshgrid(*[np.arange(0, c, 2) for c in counts], indexing="ij"), -1)
    refs = refs.reshape(-1, len(shape)).astype(np.int32)
    vg = _match_volume(cuda, native, vol, block, radius, max_m, 2, thr, _abi.MATCH_EXACT, refs=refs)
    patches, pc = _patch_table(vol, block)
    assert tuple(pc) == counts
    pg = gpu_match_patches(cuda, native, patches, counts, refs, radius, max_m, 2, thr, DEV)
    np.testing.assert_array_equal(vg[1], pg[1])
    np.testing.assert_array_equal(vg[2], pg[2])
    np.testing.assert_array_equal(vg[0], pg[0])


def _match_volume_ssd(cuda, native, vol, block, radius, max_m, min_m, thr, precision, noise=None, gamma=0.0):
    """SSD matching of a volume (every second position as reference), plain or
    with the noise-bias table ``noise`` over the search offsets."""
    from bmnd_gb300 import _abi

    shape = vol.shape
    counts = tuple(s - b + 1 for s, b in zip(shape, block))
    refs = np.stack(np.meshgrid(*[np.arange(0, c, 2) for c in counts], indexing="ij"), -1)
    refs = refs.reshape(-1, len(shape)).astype(np.int32)
    dev = cuda.device("cuda:0")
    vt = cuda.from_numpy(np.ascontiguousarray(vol, dtype=np.float32)).to(dev)
    rt = cuda.from_numpy(refs).to(dev)
    n = refs.shape[0]
    tt = cuda.full((n,), float(np.float32(thr)), device=dev)
    sel = cuda.full((n, max_m), -7, dtype=cuda.int32, device=dev)
    cnt = cuda.full((n,), -7, dtype=cuda.int32, device=dev)
    acc = cuda.full((n,), -7, dtype=cuda.int32, device=dev)
    p = _mp(counts, radius, max_m, min_m, SSD, stabilize=False)
    p.precision = precision
    sh = (ctypes.c_int32 * len(shape))(*shape)
    bl = (ctypes.c_int32 * len(shape))(*block)
    if noise is None:
        _abi.check(native.bmnd_blockmatch_volume(ctypes.byref(p), vt.data_ptr(), sh, bl, rt.data_ptr(), n,
                                                 tt.data_ptr(), sel.data_ptr(), cnt.data_ptr(), acc.data_ptr(), 0))
    else:
        nt = cuda.from_numpy(np.ascontiguousarray(noise, dtype=np.float32)).to(dev)
        _abi.check(native.bmnd_blockmatch_volume_biased(ctypes.byref(p), vt.data_ptr(), sh, bl, rt.data_ptr(), n,
                                                        tt.data_ptr(), nt.data_ptr(), float(gamma), sel.data_ptr(),
                                                        cnt.data_ptr(), acc.data_ptr(), 0))
    cuda.cuda.synchronize()
    return sel.cpu().numpy(), cnt.cpu().numpy(), acc.cpu().numpy()


@pytest.mark.parametrize("shape,block,radius,max_m,thr_frac,kind", [
    ((72, 80), (8, 8), (19, 19), 32, 0.4, "smooth"),
    ((64, 72), (8, 8), (19, 19), 16, 3.0, "noise"),
    ((60, 64), (8, 8), (19, 19), 32, 0.02, "flat"),
    ((30, 34, 38), (5, 5, 5), (7, 7, 7), 32, 0.8, "smooth"),
    ((32, 30, 36), (4, 4, 4), (7, 7, 7), 16, 3.0, "noise"),
    ((26, 28, 30), (5, 5, 5), (7, 7, 7), 32, 0.8, "large"),
    ((28, 30, 26), (4, 4, 4), (7, 7, 7), 16, 0.05, "offset"),
    ((64, 60), (8, 8), (19, 19), 32, 0.05, "offset"),
])
@pytest.mark.parametrize("bias", [False, True])
def test_tensor_core_ssd_matching_equals_exact(cuda, native, shape, block, radius, max_m, thr_frac, kind, bias):
    """SSD matching with the BF16 tensor-core screening and exact float32
    rescoring (precision fast) gives the exact kernel's match tables and
    accepted counts bit for bit, with and without the noise-bias correction."""
    from bmnd_gb300 import _abi

    rng = np.random.default_rng(zlib.crc32(repr((shape, kind, bias)).encode()))
    grids = np.meshgrid(*[np.linspace(0, 1, s) for s in shape], indexing="ij")
    smooth = 5.0 + 20.0 * np.sin(3 * grids[0]) ** 2 + 10.0 * grids[-1]
    if kind == "smooth":
        vol = smooth + rng.normal(0, 1.0, size=shape)
    elif kind == "noise":
        vol = rng.normal(10.0, 3.0, size=shape)
    elif kind == "large":
        vol = 2000.0 + 50.0 * smooth + rng.normal(0, 5.0, size=shape)
    elif kind == "offset":  # a denoised estimate far from zero: small distances under large norms
        vol = 3000.0 + 0.2 * smooth + rng.normal(0, 0.01, size=shape)
    else:
        vol = np.full(shape, 7.25) + (rng.random(shape) < 0.02) * 3.0
    vol = vol.astype(np.float32)
    span = float(vol.max() - vol.min())
    P = int(np.prod(block))
    thr = thr_frac * P * (span / 8.0) ** 2
    noise = gamma = None
    if bias:
        noise = rng.uniform(0.0, 2.0, size=tuple(2 * r + 1 for r in radius)).reshape(-1) * P
        gamma = 1.5
    args = (cuda, native, vol, block, radius, max_m, 2, thr)
    ex = _match_volume_ssd(*args, _abi.MATCH_EXACT, noise=noise, gamma=gamma or 0.0)
    tc = _match_volume_ssd(*args, _abi.MATCH_FAST, noise=noise, gamma=gamma or 0.0)
    np.testing.assert_array_equal(tc[1], ex[1])
    np.testing.assert_array_equal(tc[2], ex[2])
    np.testing.assert_array_equal(tc[0], ex[0])
