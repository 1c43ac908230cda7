"""Hamming k = 2 matching (Matcher::KnnMatch, src/Matcher.cpp:245-302).

CPU: the oracle against the reference's loop written out in Python on small
sets (ties, fewer than two train descriptors, the filters).  GPU: the kernel
against the oracle, bit-exact on indices, distances and keep flags, over
sizes that exercise partial query blocks and several train chunks."""
import numpy as np
import pytest

from mcvslam_gb300 import synth
from oracle import oracle


def _loop_knn(q, t, ratio, max_dist):
    """The reference's per-query scan (src/Matcher.cpp:255-279) and the two
    filters (src/Matcher.cpp:23-34,100-111) as plain Python."""
    nq = q.shape[0]
    idx = np.zeros((nq, 2), np.int32)
    dist = np.zeros((nq, 2), np.int32)
    keep = np.zeros(nq, np.uint8)
    for i in range(nq):
        d = [999, 999]
        ix = [0, 0]
        for j in range(t.shape[0]):
            dd = int(np.unpackbits(q[i] ^ t[j]).sum())
            if dd < d[0]:
                d[1], ix[1] = d[0], ix[0]
                d[0], ix[0] = dd, j
            elif dd < d[1]:
                d[1], ix[1] = dd, j
        idx[i] = ix
        dist[i] = d
        r = np.float32(d[0]) / np.float32(d[1]) if d[1] else np.float32(np.nan)
        keep[i] = 1 if (r <= np.float32(ratio) and d[0] <= max_dist) else 0
    return idx, dist, keep


def _tie_sets(seed, nq, nt, alphabet=4):
    # descriptors drawn from a small alphabet: many equal distances
    rng = np.random.default_rng(seed)
    base = rng.integers(0, 256, size=(alphabet, 32), dtype=np.uint8)
    return base[rng.integers(0, alphabet, nq)], base[rng.integers(0, alphabet, nt)]


@pytest.mark.parametrize("nq,nt,seed", [(20, 50, 1), (7, 0, 2), (9, 1, 3), (5, 2, 4), (0, 10, 5)])
def test_oracle_equals_reference_loop(nq, nt, seed):
    q, t = synth.descriptors(nq, nt, seed)
    for ratio, md in ((0.6, 46), (0.8, 100)):
        got = oracle.knn_hamming(q, t, ratio, md)
        want = _loop_knn(q, t, ratio, md)
        for g, w in zip(got, want):
            np.testing.assert_array_equal(g, w)


def test_oracle_ties_and_threads():
    q, t = _tie_sets(6, 30, 40)
    want = _loop_knn(q, t, 0.6, 46)
    for nth in (1, 4):
        got = oracle.knn_hamming(q, t, 0.6, 46, n_threads=nth)
        for g, w in zip(got, want):
            np.testing.assert_array_equal(g, w)
    # equal descriptors: d0 == 0, d1 == 0 -> ratio 0/0 is NaN, dropped
    same = np.zeros((2, 32), np.uint8)
    idx, dist, keep = oracle.knn_hamming(same[:1], same, 0.6, 46)
    assert list(idx[0]) == [0, 1] and list(dist[0]) == [0, 0] and keep[0] == 0


GPU_CASES = [
    (1, 1, 11), (1, 0, 12), (3, 2, 13), (129, 700, 14), (2000, 2000, 15), (37, 20000, 16), (5000, 300, 17),
    (1000, 65536, 18),
]


@pytest.mark.gpu
@pytest.mark.parametrize("nq,nt,seed", GPU_CASES)
def test_gpu_matches_oracle(gpu, nq, nt, seed):
    from mcvslam_gb300 import matcher

    q, t = synth.descriptors(nq, nt, seed)
    idx, dist, keep, ms = matcher.knn_hamming(q, t)
    oi, od, ok = oracle.knn_hamming(q, t, n_threads=8)
    np.testing.assert_array_equal(idx, oi)
    np.testing.assert_array_equal(dist, od)
    np.testing.assert_array_equal(keep, ok)
    assert ms >= 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("nq,nt,seed", [(300, 5000, 21), (1, 3, 22), (130, 1030, 23)])
def test_gpu_ties_resolve_to_smaller_index(gpu, nq, nt, seed):
    from mcvslam_gb300 import matcher

    q, t = _tie_sets(seed, nq, nt)
    got = matcher.knn_hamming(q, t, 0.8, 100)[:3]
    want = oracle.knn_hamming(q, t, 0.8, 100, n_threads=8)
    for g, w in zip(got, want):
        np.testing.assert_array_equal(g, w)


@pytest.mark.gpu
def test_gpu_device_entry_on_torch_stream(gpu):
    import torch

    from mcvslam_gb300 import matcher

    q, t = synth.descriptors(3000, 9000, 31)
    dq = torch.from_numpy(q).cuda()
    dt = torch.from_numpy(t).cuda()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        idx, dist, keep = matcher.knn_hamming_device(dq, dt, 0.7, 60)
    s.synchronize()
    oi, od, ok = oracle.knn_hamming(q, t, 0.7, 60, n_threads=8)
    np.testing.assert_array_equal(idx.cpu().numpy(), oi)
    np.testing.assert_array_equal(dist.cpu().numpy(), od)
    np.testing.assert_array_equal(keep.cpu().numpy(), ok)
