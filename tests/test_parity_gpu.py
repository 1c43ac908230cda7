"""GPU solver vs the CPU oracle through the C ABI.

FP64 plain mode must follow g2o's LM trial by trial: chi2 within 1e-9
relative, the same accept/reject decisions and lambda sequence, final poses
within 1e-8 m / 1e-8 rad.  Mixed precision must end within 1e-6 relative of
the FP64 final cost (evaluated in FP64)."""
import numpy as np
import pytest

from mcvslam_gb300 import ba, synth
from oracle import oracle

pytestmark = pytest.mark.gpu

CHI_RTOL = 1e-9
POSE_TOL_M = 1e-8
POSE_TOL_RAD = 1e-8


def rot_diff(qa, qb):
    """Angle (rad) between two unit quaternions (x y z w): 2 atan2(|vec|, |w|) of qa * conj(qb)."""
    va, vb = np.asarray(qa[:3]), np.asarray(qb[:3])
    w = qa[3] * qb[3] + va @ vb
    v = qb[3] * va - qa[3] * vb - np.cross(va, vb)
    return 2 * np.arctan2(np.linalg.norm(v), abs(w))


def compare_logs(g, o):
    assert len(g) == len(o), (len(g), len(o))
    for a, b in zip(g, o):
        assert (a["iteration"], a["trial"], a["accepted"], a["solve_ok"]) == \
               (b["iteration"], b["trial"], b["accepted"], b["solve_ok"])
        for k in ("chi_before", "chi_after", "lambda", "scale"):
            assert abs(a[k] - b[k]) <= CHI_RTOL * abs(b[k]), (k, a, b)


def compare_state(g, o, pr, pt_tol=1e-7):
    qt, X = g["pose_qt"], g["point_X"]
    for k in range(pr.n_poses):
        assert np.abs(qt[k, 4:] - o["pose_qt"][k, 4:]).max() <= POSE_TOL_M
        assert rot_diff(qt[k, :4], o["pose_qt"][k, :4]) <= POSE_TOL_RAD
    assert np.abs(X - o["point_X"]).max() <= pt_tol


@pytest.mark.parametrize("cfg", [1, 2])
def test_fp64_follows_oracle_trial_by_trial(cfg, gpu):
    pr = synth.config(cfg)
    o = oracle.optimize(pr, 10)
    g = ba.solve(pr, 10, "fp64")
    assert g["stats"]["iterations"] == o["ret"]
    compare_logs(g["log"], o["log"])
    assert abs(g["stats"]["final_chi2"] - o["final_chi2"]) <= CHI_RTOL * o["final_chi2"]
    compare_state(g, o, pr)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_reference_style_stereo_and_fixed_points(seed, gpu):
    pr = synth.reference_style(seed)
    assert (pr.edge_type == 1).any() and pr.point_fixed.any()
    o = oracle.optimize(pr, 10)
    g = ba.solve(pr, 10, "fp64")
    compare_logs(g["log"], o["log"])
    compare_state(g, o, pr)


def test_edge_chi2_matches_oracle(gpu):
    pr = synth.reference_style(7)
    o = oracle.optimize(pr, 5)
    with ba.Solver() as s:
        s.load(pr)
        s.optimize(5)
        chi2 = s.edge_chi2()
    np.testing.assert_allclose(chi2, o["edge_chi2"], rtol=1e-8, atol=1e-9)


def test_pose_only_rounds_match_oracle(gpu):
    pr = synth.pose_only(800, seed=41)
    o = oracle.pose_optimization(pr, rounds=4, iters=10, chi2_thr=5.991)
    with ba.Solver() as s:
        s.load(pr)
        inl, written = s.pose_optimization(4, 10, 5.991, 2)
        lv = s.levels()
        qt, _ = s.state()
    assert inl == o["ret"] and written == o["pose_written"]
    np.testing.assert_array_equal(lv, o["edge_level"])
    assert np.abs(qt[0, 4:] - o["pose_qt"][0, 4:]).max() <= POSE_TOL_M
    assert rot_diff(qt[0, :4], o["pose_qt"][0, :4]) <= POSE_TOL_RAD


def _unary_problem(name):
    """EdgeSE3XYZ2CameraOnlyPose (include/OptimizeTypes.hpp:20-68) problems:
    every edge unary (the point is a constant of the edge), or every ninth
    edge of config 1 unary beside binary edges."""
    if name == "unary":
        pr = synth.pose_only(800, seed=5)
        pr.edge_type[:] = synth.EDGE_UNARY
        return pr
    pr = synth.config(1)
    pr.edge_type[::9] = synth.EDGE_UNARY
    return pr


@pytest.mark.parametrize("name,iters", [("unary", 4), ("mixed_types", 10)])
def test_unary_edges_follow_oracle_trial_by_trial(name, iters, gpu):
    """Unary edges build their 6x6 pose block and b_p term only
    (base_unary_edge.hpp:51-79); FP64 plain follows the oracle trial by trial.
    The single-pose problem has converged to the last bits after about five
    iterations; beyond that the gain ratio of a trial is rounding noise
    (|rho| ~ 1e-8 on a cost change of 1e-10) and the accept/reject decision is
    not a property of the algorithm, so it is compared over four."""
    pr = _unary_problem(name)
    o = oracle.optimize(pr, iters)
    g = ba.solve(pr, iters, "fp64")
    assert g["stats"]["iterations"] == o["ret"]
    compare_logs(g["log"], o["log"])
    assert abs(g["stats"]["final_chi2"] - o["final_chi2"]) <= CHI_RTOL * o["final_chi2"]
    compare_state(g, o, pr)


def test_unary_pose_only_rounds_match_oracle(gpu):
    """PoseOptimization's four rounds (src/PoseEstimation.cpp:48-130) over unary
    edges: inlier count, written flag, per-edge levels and the final pose."""
    pr = synth.pose_only(1200, seed=43)
    pr.edge_type[:] = synth.EDGE_UNARY
    o = oracle.pose_optimization(pr, rounds=4, iters=10, chi2_thr=5.991)
    with ba.Solver() as s:
        s.load(pr)
        inl, written = s.pose_optimization(4, 10, 5.991, 2)
        lv = s.levels()
        qt, _ = s.state()
    assert inl == o["ret"] and written == o["pose_written"]
    np.testing.assert_array_equal(lv, o["edge_level"])
    assert np.abs(qt[0, 4:] - o["pose_qt"][0, 4:]).max() <= POSE_TOL_M
    assert rot_diff(qt[0, :4], o["pose_qt"][0, :4]) <= POSE_TOL_RAD


def test_local_ba_filter_matches_oracle(gpu):
    pr = synth.config(1)
    o = oracle.local_ba(pr, 10)
    with ba.Solver() as s:
        s.load(pr)
        succ, written = s.local_ba(10, 5.991)
        lv = s.levels()
    assert succ == o["ret"] and written == o["written"]
    np.testing.assert_array_equal(lv, o["edge_level"])


@pytest.mark.parametrize("cfg,iters", [(1, 10), (2, 10), (2, 20), (5, 20)])
def test_mixed_precision_final_cost_gap(cfg, iters, gpu):
    """Final cost of the mixed-precision solve, evaluated in FP64, within 1e-6
    (either side) of the FP64 solve after the same iterations.  The FP32 point
    blocks are carried as float-float pairs and inverted in FP64: rounded to
    single FP32 entries they moved the config-2 path by 6e-6 at 10 iterations
    (the inverse of an ill-conditioned 3x3 block enlarges their rounding)."""
    pr = synth.config(cfg)
    plain = ba.solve(pr, iters, "fp64")
    mixed = ba.solve(pr, iters, "mixed")
    # FP64 cost of the mixed-precision result
    with ba.Solver() as s:
        s.load(pr)
        s.set_state(mixed["pose_qt"], mixed["point_X"])
        st = s.optimize(0)
    chi_mixed = st["initial_chi2"]
    chi_plain = plain["stats"]["final_chi2"]
    gap = (chi_mixed - chi_plain) / chi_plain
    assert abs(gap) <= 1e-6, gap
    terr = np.abs(mixed["pose_qt"][:, 4:] - plain["pose_qt"][:, 4:]).max()
    assert terr < 1e-3


def test_solves_are_deterministic(gpu):
    pr = synth.config(1)
    a = ba.solve(pr, 10, "fp64")
    b = ba.solve(pr, 10, "fp64")
    np.testing.assert_array_equal(a["pose_qt"], b["pose_qt"])
    np.testing.assert_array_equal(a["point_X"], b["point_X"])


def test_points_only_problem(gpu):
    pr = synth.config(1)
    pr.pose_fixed[:] = 1
    o = oracle.optimize(pr, 5)
    g = ba.solve(pr, 5, "fp64")
    compare_logs(g["log"], o["log"])
    assert np.abs(g["point_X"] - o["point_X"]).max() <= 1e-8


def test_poses_only_problem(gpu):
    pr = synth.config(1)
    pr.point_fixed[:] = 1
    o = oracle.optimize(pr, 5)
    g = ba.solve(pr, 5, "fp64")
    compare_logs(g["log"], o["log"])
    compare_state(g, o, pr)


def test_zero_iterations_returns_initial_cost(gpu):
    pr = synth.config(1)
    with ba.Solver() as s:
        s.load(pr)
        st = s.optimize(0)
    o = oracle.optimize(pr, 1)
    assert abs(st["initial_chi2"] - o["log"][0]["chi_before"]) <= CHI_RTOL * o["log"][0]["chi_before"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_and_host_driven_loops_agree(precision, gpu):
    pr = synth.config(1)
    a = ba.solve(pr, 10, precision, use_graph=True)
    b = ba.solve(pr, 10, precision, use_graph=False)
    np.testing.assert_array_equal(a["pose_qt"], b["pose_qt"])
    np.testing.assert_array_equal(a["point_X"], b["point_X"])
    assert len(a["log"]) == len(b["log"])
    np.testing.assert_array_equal(a["log"]["chi_after"], b["log"]["chi_after"])


def test_prepared_solve_repeats_from_the_initial_state(gpu):
    pr = synth.config(1)
    ref = ba.solve(pr, 10, "mixed")
    with ba.Solver(precision="mixed") as s:
        s.load(pr)
        s.prepare()
        st1 = s.solve_prepared(10)
        st2 = s.solve_prepared(10)
        s.fetch_state()
        qt, X = s.state()
    assert st1["final_chi2"] == st2["final_chi2"] == ref["stats"]["final_chi2"]
    assert st1["h2d_bytes"] == 0
    np.testing.assert_array_equal(qt, ref["pose_qt"])
    np.testing.assert_array_equal(X, ref["point_X"])


def test_profiled_run_reports_every_phase(gpu):
    pr = synth.config(1)
    with ba.Solver(precision="mixed", profile=True) as s:
        s.load(pr)
        st = s.optimize(5)
    assert all(n > 0 for n in st["n_phase"])
    assert st["kernel_launches"] > 0 and st["ms_phase"][0] > 0


def _solve_both(pr, iters, precision):
    out = []
    for host in (True, False):
        with ba.Solver(precision=precision, device=0, host_structure=host) as s:
            s.load(pr)
            st = s.optimize(iters)
            qt, X = s.state()
            out.append((st, s.trial_log(), qt, X))
    return out


def _problems():
    c1 = synth.config(1)
    lv = c1.copy()
    lv.edge_level[::7] = 1                      # inactive edges
    fx = c1.copy()
    fx.point_fixed[::5] = 1                     # fixed points: edges without a free point
    fx.pose_fixed[:3] = 1                       # and edges with every vertex fixed
    un = synth.pose_only(800, seed=5)
    un.edge_type[:] = synth.EDGE_UNARY         # unary edges with constant points
    mx = c1.copy()
    mx.edge_type[::9] = synth.EDGE_UNARY       # unary and binary edges together
    return [("config1", c1), ("levels", lv), ("fixed", fx), ("stereo", synth.reference_style(3)),
            ("pose_only", synth.pose_only(800, seed=5)), ("unary", un), ("mixed_types", mx)]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_device_structure_equals_host_structure(precision, gpu):
    """The structure compiled on the device gives bit-identical solves."""
    for name, pr in _problems():
        (sh, lh, qh, xh), (sd, ld, qd, xd) = _solve_both(pr, 6, precision)
        for k in ("n_active_edges", "n_free_poses", "n_free_points", "iterations", "trials"):
            assert sh[k] == sd[k], (name, k, sh[k], sd[k])
        assert sh["final_chi2"] == sd["final_chi2"], name
        np.testing.assert_array_equal(lh, ld, err_msg=name)
        np.testing.assert_array_equal(qh, qd, err_msg=name)
        np.testing.assert_array_equal(xh, xd, err_msg=name)


def test_cached_workspaces_give_identical_solves(gpu):
    """Handles reuse the workspace of destroyed ones (buffers, staging, graph):
    a solve after a differently sized one equals a solve on a fresh workspace."""
    from mcvslam_gb300 import _native

    a, b = synth.config(1), synth.reference_style(2)

    def run(pr):
        with ba.Solver(precision="mixed", device=0) as s:
            s.load(pr)
            st = s.optimize(5)
            return st["final_chi2"], s.trial_log(), s.state()

    _native.lib().mcba_release_cached(-1)
    first = run(a)
    run(b)
    run(a)
    again = run(a)
    _native.lib().mcba_release_cached(0)
    fresh = run(a)
    for other in (again, fresh):
        assert other[0] == first[0]
        np.testing.assert_array_equal(other[1], first[1])
        np.testing.assert_array_equal(other[2][0], first[2][0])
        np.testing.assert_array_equal(other[2][1], first[2][1])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_indefinite_reduced_system_follows_oracle(precision, gpu):
    """Every edge of one free keyframe carries a negative information weight,
    so the reduced camera system is indefinite until the damping outgrows it:
    the first trials' factorisations meet a negative pivot (g2o's solve() ==
    false, chi2_new = DBL_MAX) and are rejected, then the growing lambda makes
    the system positive definite and the solve proceeds -- trial by trial as
    the oracle (FP64), with the same accept/fail pattern (mixed)."""
    pr = synth.config(1)
    pr.edge_info[pr.edge_pose == 5] = -1.0
    o = oracle.optimize(pr, 3)
    with ba.Solver(precision=precision) as s:
        s.load(pr)
        s.optimize(3)
        log = s.trial_log()
    assert (~o["log"]["solve_ok"].astype(bool)).sum() >= 3
    np.testing.assert_array_equal(log["solve_ok"], o["log"]["solve_ok"])
    np.testing.assert_array_equal(log["accepted"], o["log"]["accepted"])
    if precision == "fp64":
        compare_logs(log, o["log"])


@pytest.mark.parametrize("n_kf", [42, 66])
def test_cluster_solve_up_to_its_largest_size_follows_oracle(n_kf, gpu):
    # 40 and 64 free keyframes: reduced systems of 240 and 384 unknowns (15 and
    # 24 tile rows, the largest the cluster factorisation takes), where the
    # backward solve holds only part of the rows in shared memory at a time;
    # corridor layout, so the reduced matrix has absent blocks
    pr = synth.local_ba(n_kf, n_kf * 60, seed=78, corridor=True)
    o = oracle.optimize(pr, 5)
    g = ba.solve(pr, 5, "fp64")
    assert g["stats"]["iterations"] == o["ret"]
    compare_logs(g["log"], o["log"])
    compare_state(g, o, pr)


def test_config5_fp64_follows_oracle_trial_by_trial(gpu):
    """The large map (300 keyframes, 200k points, 1.6M edges): a reduced
    camera system of 1788 unknowns through the tiled factorisation, three LM
    iterations trial by trial against the multi-threaded oracle."""
    import os

    pr = synth.config(5)
    o = oracle.optimize(pr, 3, n_threads=os.cpu_count() or 1)
    g = ba.solve(pr, 3, "fp64")
    assert g["stats"]["n_free_poses"] * 6 == 1788
    assert g["stats"]["iterations"] == o["ret"]
    compare_logs(g["log"], o["log"])
    assert abs(g["stats"]["final_chi2"] - o["final_chi2"]) <= CHI_RTOL * o["final_chi2"]
    compare_state(g, o, pr)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_large_corridor_window_uses_tiled_solve_and_follows_oracle(precision, gpu):
    # 70 free keyframes (reduced system 420 > 384: the tiled factorisation),
    # corridor layout so many keyframe pairs share no point: the reduced
    # matrix has absent blocks, which every trial must see as zeros again
    pr = synth.local_ba(72, 72 * 60, seed=77, corridor=True)
    o = oracle.optimize(pr, 6)
    g = ba.solve(pr, 6, precision)
    if precision == "fp64":
        assert g["stats"]["iterations"] == o["ret"]
        compare_logs(g["log"], o["log"])
        compare_state(g, o, pr)
    else:
        assert abs(g["stats"]["final_chi2"] - o["final_chi2"]) <= 1e-4 * o["final_chi2"]
