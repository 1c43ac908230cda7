"""Stereo matching (Frame::ComputeStereoMatch, src/Frame.cpp:150-325).

CPU: the oracle against the reference's function written out in Python on
small batches, and the host-side validation of the C entry.  GPU: the
kernels against the oracle, bit-exact on u_right and depth."""
import math

import numpy as np
import pytest

from mcvslam_gb300 import synth
from oracle import oracle

F32 = np.float32


def _loop_stereo(sb):
    """The reference's loop in Python, float32 through numpy scalars."""
    nl_all = int(sb.left_begin[-1])
    u_right = np.full(nl_all, -1, np.float32)
    depth = np.full(nl_all, -1, np.float32)
    for f in range(sb.n_frames):
        l0, l1 = int(sb.left_begin[f]), int(sb.left_begin[f + 1])
        r0, r1 = int(sb.right_begin[f]), int(sb.right_begin[f + 1])
        rows = [[] for _ in range(sb.image_rows)]
        for iR in range(r1 - r0):
            y = F32(sb.right_xy[r0 + iR, 1])
            r = F32(10.0) * F32(sb.scale[sb.right_oct[r0 + iR]])
            for yi in range(max(math.floor(y - r), 0), min(math.ceil(y + r), sb.image_rows - 1) + 1):
                rows[yi].append(iR)
        maxD = min(F32(sb.bf) / F32(sb.b), F32(1000.0))
        minD = F32(1.0)
        pairs = []
        for iL in range(l1 - l0):
            lev = int(sb.left_oct[l0 + iL])
            uL, vL = F32(sb.left_xy[l0 + iL, 0]), F32(sb.left_xy[l0 + iL, 1])
            if not (0 <= vL < sb.image_rows):
                continue
            cands = rows[int(vL)]
            if not cands:
                continue
            minU, maxU = uL - maxD, uL - minD
            if maxU < 0:
                continue
            cand = [iR for iR in cands if lev - 1 <= sb.right_oct[r0 + iR] <= lev + 1
                    and minU <= sb.right_xy[r0 + iR, 0] <= maxU]
            if not cand:
                continue
            d, di = [999, 999], [0, 0]
            for j, iR in enumerate(cand):
                dj = int(np.unpackbits(sb.left_desc[l0 + iL] ^ sb.right_desc[r0 + iR]).sum())
                if dj < d[0]:
                    d[1], di[1] = d[0], di[0]
                    d[0], di[0] = dj, j
                elif dj < d[1]:
                    d[1], di[1] = dj, j
            if not (F32(d[0]) / F32(d[1]) <= F32(0.70)) or d[0] > 34:
                continue
            uR0 = F32(sb.right_xy[r0 + cand[di[0]], 0])
            sf = F32(sb.inv_scale[lev])
            rnd = lambda x: F32(math.floor(float(x) + 0.5)) if x >= 0 else F32(-math.floor(-float(x) + 0.5))  # noqa
            suL, svL, suR0 = rnd(uL * sf), rnd(vL * sf), rnd(uR0 * sf)
            R, C = int(sb.level_rows[lev]), int(sb.level_cols[lev])
            if svL - 5 < 0 or svL + 6 >= R or suL - 5 < 0 or suL + 6 >= C:
                continue
            off = int(sb.level_offset[lev])
            imL = sb.left_pyr[f, off:off + R * C].reshape(R, C).astype(np.int32)
            imR = sb.right_pyr[f, off:off + R * C].reshape(R, C).astype(np.int32)
            y, xl, xr = int(svL), int(suL), int(suR0)
            if suR0 < 0 or suR0 + 11 >= C or xr - 10 < 0:
                continue
            IL = imL[y - 5:y + 6, xl - 5:xl + 6]
            IL = IL - IL[5, 5]
            dists = []
            for inc in range(-5, 6):
                IR = imR[y - 5:y + 6, xr + inc - 5:xr + inc + 6]
                IR = IR - IR[5, 5]
                dists.append(int(np.abs(IL - IR).sum()))
            best = min(range(11), key=lambda k: (dists[k], k))
            if best in (0, 10):
                continue
            d1, d2, d3 = F32(dists[best - 1]), F32(dists[best]), F32(dists[best + 1])
            delta = (d1 - d3) / (F32(2.0) * (d1 + d3 - F32(2.0) * d2))
            if delta < -1 or delta > 1:
                continue
            buR = F32(sb.scale[lev]) * ((F32(suR0) + F32(best - 5)) + delta)
            disp = uL - buR
            if minD <= disp < maxD:
                depth[l0 + iL] = F32(sb.bf) / disp
                u_right[l0 + iL] = buR
                pairs.append((dists[best], iL))
        if not pairs:
            continue
        pairs.sort()
        med = F32(pairs[len(pairs) // 2][0])
        th_max, th_min = F32(1.6) * med, F32(0.4 * float(med))
        for dist, iL in pairs:
            if F32(dist) > th_max or F32(dist) < th_min:
                u_right[l0 + iL] = -1
                depth[l0 + iL] = -1
    return u_right, depth


@pytest.mark.parametrize("seed", [1, 2])
def test_oracle_equals_reference_loop(seed):
    sb = synth.stereo_batch(2, 120, 40, seed)
    u, d = oracle.stereo_match(sb)
    pu, pd = _loop_stereo(sb)
    np.testing.assert_array_equal(u, pu)
    np.testing.assert_array_equal(d, pd)
    assert (u >= 0).sum() > 30


def test_oracle_threads_agree():
    sb = synth.stereo_batch(6, 300, 100, 3)
    a = oracle.stereo_match(sb)
    b = oracle.stereo_match(sb, n_threads=4)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


def test_host_validation_without_device():
    from mcvslam_gb300 import _native as N
    from mcvslam_gb300 import matcher

    sb = synth.stereo_batch(1, 20, 5, 4)
    sb.left_oct[3] = 8
    with pytest.raises(N.MCBAError) as e:
        matcher.stereo_match(sb)
    assert e.value.status == 1
    sb = synth.stereo_batch(1, 20, 5, 4)
    sb.image_rows = 9000
    with pytest.raises(N.MCBAError) as e:
        matcher.stereo_match(sb)
    assert e.value.status == 9
    sb = synth.stereo_batch(1, 20, 5, 4)
    sb.right_xy[2, 1] = np.inf
    with pytest.raises(N.MCBAError) as e:
        matcher.stereo_match(sb)
    assert e.value.status == 4


@pytest.mark.gpu
@pytest.mark.parametrize("F,nl,nc,seed", [(1, 50, 10, 11), (4, 1500, 500, 12), (16, 800, 300, 13), (3, 2000, 0, 14)])
def test_gpu_matches_oracle(gpu, F, nl, nc, seed):
    from mcvslam_gb300 import matcher

    sb = synth.stereo_batch(F, nl, nc, seed)
    u, d, ms = matcher.stereo_match(sb)
    ou, od = oracle.stereo_match(sb, n_threads=8)
    np.testing.assert_array_equal(u, ou)
    np.testing.assert_array_equal(d, od)
    assert (u >= 0).sum() > 0


@pytest.mark.gpu
def test_gpu_frames_without_matches(gpu):
    from mcvslam_gb300 import matcher

    sb = synth.stereo_batch(4, 300, 50, 21)
    # frame 1 loses its right keypoints, frame 2 its left keypoints
    keep_r = np.r_[0:sb.right_begin[1], sb.right_begin[2]:sb.right_begin[4]]
    keep_l = np.r_[0:sb.left_begin[2], sb.left_begin[3]:sb.left_begin[4]]
    rb = sb.right_begin.copy()
    rb[2:] -= sb.right_begin[2] - sb.right_begin[1]
    lb = sb.left_begin.copy()
    lb[3:] -= sb.left_begin[3] - sb.left_begin[2]
    sb.right_xy, sb.right_oct, sb.right_desc = sb.right_xy[keep_r], sb.right_oct[keep_r], sb.right_desc[keep_r]
    sb.left_xy, sb.left_oct, sb.left_desc = sb.left_xy[keep_l], sb.left_oct[keep_l], sb.left_desc[keep_l]
    sb.right_begin, sb.left_begin = rb, lb
    u, d, _ = matcher.stereo_match(sb)
    ou, od = oracle.stereo_match(sb)
    np.testing.assert_array_equal(u, ou)
    np.testing.assert_array_equal(d, od)
    assert (u[lb[1]:lb[2]] == -1).all()


@pytest.mark.gpu
def test_gpu_device_entry_repeats(gpu):
    from mcvslam_gb300 import matcher

    sb = synth.stereo_batch(8, 1000, 300, 31)
    ou, od = oracle.stereo_match(sb, n_threads=8)
    db = matcher.DeviceStereoBatch(sb)
    for _ in range(3):
        u, d = db.run()
        np.testing.assert_array_equal(u.cpu().numpy(), ou)
        np.testing.assert_array_equal(d.cpu().numpy(), od)
