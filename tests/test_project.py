"""Map-point projection + windowed match (Object::ProjectBunchMapPoints,
src/Object.cpp:208-236).

CPU: the oracle against the reference's loop written out in Python on small
batches (grid, area search, k = 2 match, filters, AddMapPoint bookkeeping),
hand-made cases of the binding rules, and the host-side validation of the C
entry.  GPU: the kernels against the oracle, exact on bindings, matches and
counts."""
import math

import numpy as np
import pytest

from mcvslam_gb300 import synth
from oracle import oracle


def _f32(x):
    return np.float32(x)


def _loop_project(b):
    """The reference's per-object loop in Python (float32 via numpy scalars)."""
    kp_bind = np.array(b.kp_bind, np.int32, copy=True)
    nm = int(b.mp_begin[-1])
    mp_match = np.full(nm, -1, np.int32)
    count = np.zeros(b.n_objects, np.int32)
    for o in range(b.n_objects):
        Rt = b.obj_Rt[o]
        fx, fy, cx, cy = [_f32(v) for v in b.obj_K[o]]
        cols, rows = int(b.obj_size[o, 0]), int(b.obj_size[o, 1])
        inv_w, inv_h = 30.0 / cols, 30.0 / rows
        k0, k1 = int(b.kp_begin[o]), int(b.kp_begin[o + 1])
        grid = {}
        for i in range(k1 - k0):
            x, y = b.kp_xy[k0 + i]
            px = math.floor(float(x) * inv_w + 0.5) if float(x) >= 0 else -math.floor(-float(x) * inv_w + 0.5)
            py = math.floor(float(y) * inv_h + 0.5) if float(y) >= 0 else -math.floor(-float(y) * inv_h + 0.5)
            if 0 <= px < 30 and 0 <= py < 30:
                grid.setdefault((px, py), []).append(i)
        bind = kp_bind[k0:k1]
        mp2idx = {int(v): i for i, v in enumerate(bind) if v >= 0}
        for m in range(int(b.mp_begin[o]), int(b.mp_begin[o + 1])):
            X = b.mp_X[m]
            Pc = [_f32(sum(float(Rt[3 * r + k]) * float(X[k]) for k in range(3)) + float(Rt[9 + r])) for r in range(3)]
            if Pc[2] < 0:
                continue
            with np.errstate(divide="ignore", invalid="ignore"):
                u = fx * Pc[0] / Pc[2] + cx
                v = fy * Pc[1] / Pc[2] + cy
            rad = _f32(b.obj_radius[o]) * _f32(b.obj_scale[o, b.mp_level[m]])
            cand = []
            if not (u < 0 or v < 0 or u >= cols or v >= rows or np.isnan(u) or np.isnan(v)):
                minx = max(0, math.floor(float(u - rad) * inv_w))
                maxx = min(29, math.ceil(float(u + rad) * inv_w))
                miny = max(0, math.floor(float(v - rad) * inv_h))
                maxy = min(29, math.ceil(float(v + rad) * inv_h))
                for ix in range(minx, maxx + 1):
                    for iy in range(miny, maxy + 1):
                        for i in grid.get((ix, iy), []):
                            dx = b.kp_xy[k0 + i, 0] - u
                            dy = b.kp_xy[k0 + i, 1] - v
                            if abs(dx) < rad and abs(dy) < rad:
                                cand.append(i)
            if not cand:
                continue
            d, di = [999, 999], [0, 0]
            for j, i in enumerate(cand):
                dj = int(np.unpackbits(b.mp_desc[m] ^ b.kp_desc[k0 + i]).sum())
                if dj < d[0]:
                    d[1], di[1] = d[0], di[0]
                    d[0], di[0] = dj, j
                elif dj < d[1]:
                    d[1], di[1] = dj, j
            if not (_f32(d[0]) / _f32(d[1]) <= _f32(b.ratio)) or d[0] > b.max_dist:
                continue
            idx = cand[di[0]]
            mid = int(b.mp_id[m])
            if mid in mp2idx:
                bind[mp2idx.pop(mid)] = -1
            if bind[idx] >= 0:
                mp2idx.pop(int(bind[idx]), None)
            bind[idx] = mid
            mp2idx[mid] = idx
            mp_match[m] = idx
            count[o] += 1
    return kp_bind, mp_match, count


def _assert_same(got, want):
    for g, w, name in zip(got, want, ("kp_bind", "mp_match", "obj_count")):
        np.testing.assert_array_equal(np.asarray(g), np.asarray(w), err_msg=name)


@pytest.mark.parametrize("seed,radius", [(1, 10.0), (2, 5.0), (3, 7.0)])
def test_oracle_equals_reference_loop(seed, radius):
    b = synth.projection_batch(3, 150, 120, seed, radius=radius)
    _assert_same(oracle.project_match(b), _loop_project(b))


def _one_object(kp_xy, kp_desc, mp_X, mp_desc, kp_bind=None, mp_prev=None, radius=10.0, size=(512, 512)):
    nk, nm = len(kp_xy), len(mp_X)
    return synth.ProjectionBatch(
        obj_Rt=np.array([[1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0]], np.float32),
        obj_K=np.array([[500, 500, 256, 256]], np.float32), obj_size=np.array([size], np.int32),
        obj_radius=np.array([radius], np.float32), obj_scale=synth.scale_factors()[None, :], ratio=0.6, max_dist=46,
        kp_begin=np.array([0, nk], np.int32), kp_xy=np.array(kp_xy, np.float32).reshape(-1, 2),
        kp_desc=np.array(kp_desc, np.uint8).reshape(-1, 32),
        kp_bind=np.array(kp_bind if kp_bind is not None else [-1] * nk, np.int32),
        mp_begin=np.array([0, nm], np.int32), mp_X=np.array(mp_X, np.float32).reshape(-1, 3),
        mp_desc=np.array(mp_desc, np.uint8).reshape(-1, 32), mp_level=np.zeros(nm, np.int32),
        mp_id=np.arange(100, 100 + nm, dtype=np.int32),
        mp_prev_kp=np.array(mp_prev if mp_prev is not None else [-1] * nm, np.int32))


def _desc(bits_set):
    d = np.zeros(256, np.uint8)
    d[list(bits_set)] = 1
    return np.packbits(d)


def test_binding_rules_by_hand():
    # kp 0 at the principal point; kp 1 one pixel right; kp 2 near the right edge
    kp_xy = [[256, 256], [257, 256], [505, 256]]
    base = _desc([])
    kp_desc = [base, _desc(range(40)), base]
    # mp 0 and mp 2 both match kp 0 (the later one keeps it), mp 1 was bound to kp 1 before
    mp_X = [[0, 0, 5], [0, 0, 5], [0, 0, 5], [249 / 500 * 5, 0, 5]]
    mp_desc = [base, _desc(range(50)), base, base]
    b = _one_object(kp_xy, kp_desc, mp_X, mp_desc, kp_bind=[-1, 101, -1], mp_prev=[-1, 1, -1, -1])
    kb, mm, cnt = oracle.project_match(b)
    _assert_same((kb, mm, cnt), _loop_project(b))
    # mp 1: distances 50 (kp 0) and 10 (kp 1): 10/50 = 0.2 -> matches kp 1 again
    assert list(mm[:3]) == [0, 1, 0]
    assert kb[0] == 102 and kb[1] == 101
    # kp 2 sits at x = 505 >= 29.5 / 30 * 512: outside the grid, never a candidate
    assert mm[3] == -1 and kb[2] == -1
    assert cnt[0] == 3


def test_behind_camera_and_outside_image():
    kp_xy = [[256, 256]]
    d = _desc([])
    mp_X = [[0, 0, -5], [0, 0, 0], [10, 0, 1], [0, 0, 5]]
    b = _one_object(kp_xy, [d], mp_X, [d] * 4)
    kb, mm, cnt = oracle.project_match(b)
    _assert_same((kb, mm, cnt), _loop_project(b))
    assert list(mm) == [-1, -1, -1, 0] and kb[0] == 103


def test_host_validation_without_device():
    from mcvslam_gb300 import _native as N
    from mcvslam_gb300 import matcher

    b = synth.projection_batch(2, 50, 40, 9)
    b.mp_level[3] = 8  # outside [0, n_levels)
    with pytest.raises(N.MCBAError) as e:
        matcher.project_match(b)
    assert e.value.status == 1
    b = synth.projection_batch(2, 50, 40, 9)
    b.kp_xy[5, 0] = np.nan
    with pytest.raises(N.MCBAError) as e:
        matcher.project_match(b)
    assert e.value.status == 4
    b = synth.projection_batch(2, 50, 40, 9)
    b.mp_prev_kp[0] = 50  # beyond the object's keypoints
    with pytest.raises(N.MCBAError) as e:
        matcher.project_match(b)
    assert e.value.status == 1


GPU_CASES = [(1, 300, 200, 11, 10.0), (8, 2000, 3000, 12, 10.0), (16, 1500, 2500, 13, 5.0), (5, 40, 900, 14, 7.0),
             (64, 500, 700, 15, 10.0)]


@pytest.mark.gpu
@pytest.mark.parametrize("O,nk,nm,seed,radius", GPU_CASES)
def test_gpu_matches_oracle(gpu, O, nk, nm, seed, radius):
    from mcvslam_gb300 import matcher

    b = synth.projection_batch(O, nk, nm, seed, radius=radius)
    kb, mm, cnt, ms = matcher.project_match(b)
    _assert_same((kb, mm, cnt), oracle.project_match(b))
    assert cnt.sum() > 0


@pytest.mark.gpu
def test_gpu_edge_cases(gpu):
    from mcvslam_gb300 import matcher

    # hand-made cases through the GPU
    kp_xy = [[256, 256], [257, 256], [505, 256]]
    base = _desc([])
    b = _one_object(kp_xy, [base, _desc(range(40)), base],
                    [[0, 0, 5], [0, 0, 5], [0, 0, 5], [249 / 500 * 5, 0, 5], [0, 0, -1], [0, 0, 0]],
                    [base, _desc(range(50)), base, base, base, base], kp_bind=[-1, 101, -1],
                    mp_prev=[-1, 1, -1, -1, -1, -1])
    _assert_same(matcher.project_match(b)[:3], oracle.project_match(b))
    # empty objects between full ones, all-duplicate descriptors (ties), no previous bindings
    b = synth.projection_batch(6, 300, 400, 21)
    b.kp_desc[:] = b.kp_desc[0]
    b.mp_desc[:] = b.kp_desc[0]
    keep = [0, 2, 5]
    kb, mp = [0], [0]
    sel_k, sel_m = [], []
    for o in range(6):
        k = np.arange(b.kp_begin[o], b.kp_begin[o + 1]) if o in keep else np.arange(0)
        m = np.arange(b.mp_begin[o], b.mp_begin[o + 1]) if o in (0, 1, 5) else np.arange(0)
        sel_k.append(k)
        sel_m.append(m)
        kb.append(kb[-1] + len(k))
        mp.append(mp[-1] + len(m))
    sk, sm = np.concatenate(sel_k), np.concatenate(sel_m)
    b.kp_begin, b.mp_begin = np.array(kb, np.int32), np.array(mp, np.int32)
    b.kp_xy, b.kp_desc, b.kp_bind = b.kp_xy[sk], b.kp_desc[sk], b.kp_bind[sk]
    b.mp_X, b.mp_desc, b.mp_level, b.mp_id = b.mp_X[sm], b.mp_desc[sm], b.mp_level[sm], b.mp_id[sm]
    b.mp_prev_kp = None
    b.kp_bind[:] = -1
    got = matcher.project_match(b)[:3]
    _assert_same(got, oracle.project_match(b))
    assert got[2][0] > 0 and got[2][1] == 0 and got[2][5] > 0


@pytest.mark.gpu
def test_gpu_device_entry_repeats(gpu):
    from mcvslam_gb300 import matcher

    b = synth.projection_batch(12, 1000, 1500, 31)
    want = oracle.project_match(b)
    db = matcher.DeviceProjectionBatch(b)
    for _ in range(3):
        kb, mm, cnt = db.run()
        _assert_same((kb.cpu().numpy(), mm.cpu().numpy(), cnt.cpu().numpy()), want)
