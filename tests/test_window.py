"""Local-BA window of a new keyframe on flat map tables (Map::AddKeyFrame's
set-up, src/Map.cpp:140-145): GrabLocalMap_Mappoint, GrabAnchorKeyFrames,
ThisMapPointBeFix and BoundleAdjustment's vertex/edge insertion.

CPU: the C oracle (oracle/window_oracle.cpp) against an independent Python
restatement written from the reference's loops, on generated maps and on
hand-made cases of the rules.  GPU: mcba_local_window against the oracle,
element for element, and the window's local BA against the oracle's."""
import math

import numpy as np
import pytest

from mcvslam_gb300 import synth
from oracle import oracle

TH2D = np.float32(math.sqrt(5.99))   # BAoptimizer::thHuber2D
TH3D = np.float32(math.sqrt(7.815))  # BAoptimizer::thHuber3D


def _py_window(m, cur, hop):
    """Straight restatement with Python sets walked in sorted order."""
    def bound(mp):
        return m.mp_kf[m.mp_kf_begin[mp]:m.mp_kf_begin[mp + 1]].tolist()

    def obs(kf, obj):
        return [o for o in range(m.obs_begin[kf], m.obs_begin[kf + 1]) if m.obs_object[o] == obj]

    def ess(kf):
        return m.ess_adj[m.ess_begin[kf]:m.ess_begin[kf + 1]].tolist()

    # GrabLocalMap_Mappoint (src/Map.cpp:730-756)
    ret = set()
    for o in obs(cur, 0):
        ret.update(bound(m.obs_point[o]))
    cur_hop, h = set(ret), hop - 1
    while h > 0 and cur_hop:
        h -= 1
        nxt = set()
        for kf in sorted(cur_hop):
            for to in ess(kf):
                if to not in ret:
                    ret.add(to)
                    nxt.add(to)
        cur_hop = nxt
    ret.discard(cur)
    # GrabAnchorKeyFrames (src/Map.cpp:775-796)
    anchors = set()
    if ret:
        kmin = min(ret, key=lambda k: m.kf_id[k])
        anchors = {k for k in set(ess(kmin)) - {kmin} if m.kf_id[k] < m.kf_id[kmin]}
    local = ret | {cur}

    def be_fix(mp):  # ThisMapPointBeFix (src/PoseEstimation.cpp:153-163)
        nf = fx = 0
        for kf in bound(mp):
            if kf in local:
                nf += 1
            elif kf in anchors:
                fx += 1
        return not ((nf + 1) * 1.0 / (fx + 1) > 1.5)

    kf2id, mp2id = {}, {}
    pose_kf, pose_fixed, point_mp, point_fixed = [], [], [], []
    edges = []
    for fixed, group in ((True, sorted(anchors)), (False, sorted(local))):
        for kf in group:
            if kf not in kf2id:
                kf2id[kf] = len(kf2id)
                pose_kf.append(kf)
                pose_fixed.append(1 if (fixed or m.kf_id[kf] == 0) else 0)
            for obj in (0, 1):
                for o in obs(kf, obj):
                    mp = int(m.obs_point[o])
                    if mp not in mp2id:
                        mp2id[mp] = len(mp2id)
                        point_mp.append(mp)
                        point_fixed.append(1 if be_fix(mp) else 0)
                    ur = float(m.obs_ur[o])
                    stereo = obj == 0 and ur != -1 and ur >= 1.0
                    lv = int(m.obs_octave[o])
                    info = (m.inv_sigma2_left if obj == 0 else m.inv_sigma2_wide)[lv]
                    edges.append((1 if stereo else 0, kf2id[kf], mp2id[mp], obj, m.obs_uv[o, 0], m.obs_uv[o, 1],
                                  np.float32(ur) if stereo else np.float32(0), info,
                                  TH2D if (obj == 0 and not stereo) else TH3D))
    role = np.zeros(m.n_keyframes, np.uint8)
    for k in local:
        role[k] |= 1
    for k in anchors:
        role[k] |= 2
    return role, pose_kf, pose_fixed, point_mp, point_fixed, edges


def _check_equal(w, py):
    role, pose_kf, pose_fixed, point_mp, point_fixed, edges = py
    np.testing.assert_array_equal(w["kf_role"], role)
    np.testing.assert_array_equal(w["pose_kf"], pose_kf)
    np.testing.assert_array_equal(w["pose_fixed"], pose_fixed)
    np.testing.assert_array_equal(w["point_mp"], point_mp)
    np.testing.assert_array_equal(w["point_fixed"], point_fixed)
    assert len(w["edge_type"]) == len(edges)
    if edges:
        e = list(zip(*edges))
        np.testing.assert_array_equal(w["edge_type"], e[0])
        np.testing.assert_array_equal(w["edge_pose"], e[1])
        np.testing.assert_array_equal(w["edge_point"], e[2])
        np.testing.assert_array_equal(w["edge_cam"], e[3])
        np.testing.assert_array_equal(w["edge_obs"][:, 0], np.asarray(e[4], np.float32))
        np.testing.assert_array_equal(w["edge_obs"][:, 1], np.asarray(e[5], np.float32))
        np.testing.assert_array_equal(w["edge_obs"][:, 2], np.asarray(e[6], np.float32))
        np.testing.assert_array_equal(w["edge_info"], np.asarray(e[7], np.float32))
        np.testing.assert_array_equal(w["edge_delta"], np.asarray(e[8], np.float32))


@pytest.mark.parametrize("seed,cur,hop", [(11, -1, 1), (12, -1, 2), (13, 30, 1), (14, -1, 3)])
def test_oracle_matches_python_restatement(seed, cur, hop):
    m = synth.map_tables(48, 4000, seed)
    cur = m.n_keyframes - 1 if cur < 0 else cur
    w = oracle.local_window(m, cur, hop)
    assert w["n_local"] > 1 and len(w["edge_type"]) > 0
    _check_equal(w, _py_window(m, cur, hop))


def _tiny_map(bound, ess, kf_ids, obs_rows, n_points):
    """Hand-made map: obs_rows = [(kf, point, object, u_right, octave)]."""
    K = len(kf_ids)
    rows = sorted(obs_rows, key=lambda r: r[0])
    ob = np.zeros(K + 1, np.int32)
    for r in rows:
        ob[r[0] + 1] += 1
    ob = np.cumsum(ob).astype(np.int32)
    mb = np.zeros(n_points + 1, np.int32)
    mk = []
    for p in range(n_points):
        mk.extend(bound.get(p, []))
        mb[p + 1] = len(mk)
    eb = np.zeros(K + 1, np.int32)
    ea = []
    for k in range(K):
        ea.extend(ess.get(k, []))
        eb[k + 1] = len(ea)
    L = 4
    s2 = (1.0 / 1.2 ** (2 * np.arange(L))).astype(np.float32)
    rig = synth.reference_rig()
    return synth.MapTables(
        kf_id=np.asarray(kf_ids, np.int64), kf_Tcw=np.tile(np.eye(4, dtype=np.float32).reshape(16), (K, 1)),
        obs_begin=ob, obs_point=np.array([r[1] for r in rows], np.int32),
        obs_object=np.array([r[2] for r in rows], np.uint8),
        obs_uv=np.array([[100.0 + i, 200.0 + 2 * i] for i in range(len(rows))], np.float32),
        obs_ur=np.array([r[3] for r in rows], np.float32), obs_octave=np.array([r[4] for r in rows], np.uint8),
        mp_Xw=np.tile(np.array([0.0, 0.0, 5.0], np.float32), (n_points, 1)), mp_kf_begin=mb,
        mp_kf=np.asarray(mk, np.int32), ess_begin=eb, ess_adj=np.asarray(ea, np.int32), inv_sigma2_left=s2,
        inv_sigma2_wide=s2.copy(), K_left=rig.K[0].copy(), K_wide=rig.K[2].copy(),
        T_wide_body=rig.T_cb[2].astype(np.float32).reshape(16), bf=float(rig.bf[0]))


def _rule_map():
    """Keyframes 0..5 (ids 0, 10, 20, 30, 40, 50), the new one is 5.  Its LEFT
    points 0, 3, 5, 6 are bound to keyframes 2, 3, 4 -> window {2, 3, 4, 5};
    the smallest id there is keyframe 2, whose essential-graph neighbours 0, 1
    (older) and 3 (newer, listed twice) make anchors {0, 1}.  Fix rule:
      p0 bound to 2, 3, 4:      free 3, fix 0 -> 4/1 > 1.5: free
      p1 bound to 2, 0, 1:      free 1, fix 2 -> 2/3: fixed
      p2 bound to 2, 3, 0:      free 2, fix 1 -> 3/2 = 1.5: fixed (not > 1.5)
      p3 bound to 4:            free
      p4 seen by 5, unbound:    1/1: fixed
      p5 bound to 3, p6 to 2, 4: free
    u_right on the new keyframe's LEFT rows: -1 and 0.5 give mono edges, 1.0
    and 37 stereo edges (MIN_DISPARITY = 1)."""
    bound = {0: [2, 3, 4], 1: [2, 0, 1], 2: [2, 3, 0], 3: [4], 5: [3], 6: [2, 4]}
    ess = {2: [0, 3, 1, 3], 0: [2], 1: [2], 3: [2]}
    rows = [(5, 0, 0, -1.0, 0), (5, 3, 0, 0.5, 1), (5, 5, 0, 1.0, 2), (5, 6, 0, 37.0, 3), (5, 4, 1, -1.0, 0),
            (5, 1, 1, -1.0, 1), (0, 1, 0, 12.0, 0), (0, 0, 1, -1.0, 2), (1, 1, 0, -1.0, 0), (2, 2, 1, -1.0, 1),
            (2, 0, 0, 3.0, 0), (3, 3, 0, -1.0, 3), (4, 1, 1, -1.0, 2)]
    return _tiny_map(bound, ess, [0, 10, 20, 30, 40, 50], rows, 7)


def test_rules_on_a_hand_made_map():
    m = _rule_map()
    w = oracle.local_window(m, 5, 1)
    np.testing.assert_array_equal(w["kf_role"], [2, 2, 1, 1, 1, 1])
    np.testing.assert_array_equal(w["pose_kf"], [0, 1, 2, 3, 4, 5])
    np.testing.assert_array_equal(w["pose_fixed"], [1, 1, 0, 0, 0, 0])
    fixed = dict(zip(w["point_mp"].tolist(), w["point_fixed"].tolist()))
    assert fixed == {0: 0, 1: 1, 2: 1, 3: 0, 4: 1, 5: 0, 6: 0}
    # keyframe 5: LEFT rows in table order, then WIDE rows
    last = w["edge_pose"] == 5
    np.testing.assert_array_equal(w["edge_type"][last], [0, 0, 1, 1, 0, 0])
    np.testing.assert_array_equal(w["edge_cam"][last], [0, 0, 0, 0, 1, 1])
    np.testing.assert_array_equal(w["edge_delta"][last], [TH2D, TH2D, TH3D, TH3D, TH3D, TH3D])
    _check_equal(w, _py_window(m, 5, 1))


def test_new_keyframe_older_than_the_window_is_anchor_and_member():
    """A frame whose id is below the window's smallest is found among the
    anchors before it is added to the window (src/Map.cpp:143-144): the
    reference then adds it fixed and inserts its edges twice."""
    bound = {0: [1, 2]}
    ess = {1: [0, 2], 0: [1], 2: [1]}
    rows = [(0, 0, 0, -1.0, 0), (1, 0, 0, -1.0, 0), (2, 0, 1, -1.0, 0)]
    m = _tiny_map(bound, ess, [5, 10, 20], rows, 1)
    w = oracle.local_window(m, 0, 1)
    np.testing.assert_array_equal(w["kf_role"], [3, 1, 1])
    np.testing.assert_array_equal(w["pose_kf"], [0, 1, 2])
    np.testing.assert_array_equal(w["pose_fixed"], [1, 0, 0])
    assert (w["edge_pose"] == 0).sum() == 2
    _check_equal(w, _py_window(m, 0, 1))


def test_isolated_keyframe_has_a_window_of_itself():
    """No bound keyframes: the window is the frame alone, no anchors."""
    rows = [(1, 0, 0, -1.0, 0), (1, 1, 1, -1.0, 0)]
    m = _tiny_map({}, {}, [0, 3], rows, 2)
    w = oracle.local_window(m, 1, 1)
    np.testing.assert_array_equal(w["kf_role"], [0, 1])
    assert w["n_anchor"] == 0 and len(w["edge_type"]) == 2
    np.testing.assert_array_equal(w["point_fixed"], [1, 1])
    _check_equal(w, _py_window(m, 1, 1))


def test_window_arguments_are_validated_on_the_host():
    """Bad arguments and malformed offsets are refused before any GPU work
    (no device is needed to see the status)."""
    from mcvslam_gb300 import ba
    from mcvslam_gb300 import _native as N

    m = _rule_map()
    with ba.Solver() as s:
        for cur, hop in ((-1, 1), (6, 1), (5, 0)):
            with pytest.raises(N.MCBAError) as ei:
                s.local_window(m, cur, hop)
            assert ei.value.status == 1  # MCBA_ERR_INVALID
        bad = _rule_map()
        bad.obs_begin = bad.obs_begin.copy()
        bad.obs_begin[2], bad.obs_begin[3] = bad.obs_begin[3], bad.obs_begin[2] + 1
        with pytest.raises(N.MCBAError):
            s.local_window(bad, 5, 1)
        bad = _rule_map()
        bad.kf_id = bad.kf_id.copy()
        bad.kf_id[3] = -4
        with pytest.raises(N.MCBAError):
            s.local_window(bad, 5, 1)


# ------------------------------------------------------------------- GPU --
def _gpu_window(m, cur, hop, precision="fp64"):
    from mcvslam_gb300 import ba

    s = ba.Solver(precision=precision)
    w = s.local_window(m, cur, hop)
    return s, w


@pytest.mark.gpu
@pytest.mark.parametrize("seed,cur,hop", [(11, -1, 1), (12, -1, 2), (13, 30, 1), (14, -1, 3)])
def test_gpu_window_equals_oracle(seed, cur, hop, gpu):
    """Roles, vertex order, fix flags and -- through the per-edge chi2 at the
    loaded estimates, in edge order -- every edge of the assembled problem."""
    m = synth.map_tables(48, 4000, seed)
    cur = m.n_keyframes - 1 if cur < 0 else cur
    o = oracle.local_window(m, cur, hop)
    s, w = _gpu_window(m, cur, hop)
    try:
        np.testing.assert_array_equal(w["kf_role"], o["kf_role"])
        np.testing.assert_array_equal(w["pose_kf"], o["pose_kf"])
        np.testing.assert_array_equal(w["point_mp"], o["point_mp"])
        np.testing.assert_array_equal(w["point_fixed"], o["point_fixed"])
        assert (w["n_local"], w["n_anchor"], w["n_edges"]) == (o["n_local"], o["n_anchor"], len(o["edge_type"]))
        pr = oracle.window_problem(m, o)
        ref = oracle.optimize(pr, 0)
        np.testing.assert_allclose(s.edge_chi2(), ref["edge_chi2"], rtol=1e-9, atol=1e-12)
    finally:
        s.close()


@pytest.mark.gpu
def test_gpu_window_rules_on_hand_made_maps(gpu):
    for m, cur in ((_rule_map(), 5), (_tiny_map({0: [1, 2]}, {1: [0, 2], 0: [1], 2: [1]}, [5, 10, 20],
                                                 [(0, 0, 0, -1.0, 0), (1, 0, 0, -1.0, 0), (2, 0, 1, -1.0, 0)],
                                                 1), 0)):
        o = oracle.local_window(m, cur, 1)
        s, w = _gpu_window(m, cur, 1)
        try:
            np.testing.assert_array_equal(w["kf_role"], o["kf_role"])
            np.testing.assert_array_equal(w["pose_kf"], o["pose_kf"])
            np.testing.assert_array_equal(w["point_mp"], o["point_mp"])
            np.testing.assert_array_equal(w["point_fixed"], o["point_fixed"])
            assert w["n_edges"] == len(o["edge_type"])
        finally:
            s.close()


def _compare_logs(g, o, rtol=1e-9):
    assert len(g) == len(o), (len(g), len(o))
    for a, b in zip(g, o):
        assert (a["iteration"], a["trial"], a["accepted"], a["solve_ok"]) == \
               (b["iteration"], b["trial"], b["accepted"], b["solve_ok"])
        for k in ("chi_before", "chi_after", "lambda", "scale"):
            assert abs(a[k] - b[k]) <= rtol * abs(b[k]), (k, a, b)


@pytest.mark.gpu
def test_gpu_window_local_ba_follows_oracle(gpu):
    """The whole local BA of Map::AddKeyFrame on the GPU -- window, assembly,
    optimize(10) trial by trial, then BoundleAdjustment's chi2 filter on a
    fresh window -- against the oracle on its own assembly."""
    m = synth.map_tables(60, 6000, 21)
    cur = m.n_keyframes - 1
    o = oracle.local_window(m, cur, 1)
    pr = oracle.window_problem(m, o)
    ref_log = oracle.optimize(pr, 10)["log"]
    ref = oracle.local_ba(pr, 10, 5.991)
    s, w = _gpu_window(m, cur, 1)
    try:
        st = s.optimize(10)
        assert st["iterations"] > 0
        _compare_logs(s.trial_log(), ref_log)
    finally:
        s.close()
    s, w = _gpu_window(m, cur, 1)
    try:
        succ, written = s.local_ba(10, 5.991)
        np.testing.assert_array_equal(s.levels(), ref["edge_level"])
        assert (succ, written) == (ref["ret"], ref["written"])
    finally:
        s.close()


@pytest.mark.gpu
def test_gpu_window_rejects_out_of_range_table_entries(gpu):
    """Indices outside their tables are caught by the kernels' own bounds
    checks (the access is skipped and an error word set): the call returns
    MCBA_ERR_INVALID and the next call on good tables succeeds."""
    from mcvslam_gb300 import _native as N

    good = synth.map_tables(24, 1500, 31)
    cur = good.n_keyframes - 1
    cases = []
    b = synth.map_tables(24, 1500, 31)
    b.obs_point = b.obs_point.copy()
    b.obs_point[b.obs_begin[cur]] = b.n_points + 7          # map point out of range
    cases.append(b)
    b = synth.map_tables(24, 1500, 31)
    b.mp_kf = b.mp_kf.copy()
    b.mp_kf[:] = np.where(np.arange(len(b.mp_kf)) % 5 == 0, b.n_keyframes + 3, b.mp_kf)  # keyframe out of range
    cases.append(b)
    b = synth.map_tables(24, 1500, 31)
    b.obs_octave = np.full_like(b.obs_octave, 9)             # octave beyond the sigma tables
    cases.append(b)
    b = synth.map_tables(24, 1500, 31)
    b.obs_object = b.obs_object.copy()
    b.obs_object[b.obs_begin[cur] + 1] = 7                   # neither LEFT nor WIDE
    cases.append(b)
    from mcvslam_gb300 import ba

    for bad in cases:
        with ba.Solver() as s:
            with pytest.raises(N.MCBAError) as ei:
                s.local_window(bad, cur, 1)
            assert ei.value.status == 1
    s, w = _gpu_window(good, cur, 1)
    s.close()
    assert w["n_edges"] > 0
