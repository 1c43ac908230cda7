"""C-ABI checks that need no GPU: exported symbols, argument validation,
float<->SE3 conversions, edge bookkeeping."""
import ctypes
import os
import re

import numpy as np
import pytest

from mcvslam_gb300 import _native as N
from mcvslam_gb300 import synth
from mcvslam_gb300.ba import Solver
from oracle import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(mcba_[a-z0-9_]+)\s*\(", txt))
    return names


def test_library_exports_every_declared_symbol():
    L = N.lib()
    names = declared_symbols()
    assert len(names) > 30
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing


def test_abi_version_and_status_strings():
    L = N.lib()
    assert L.mcba_abi_version() == 1
    assert L.mcba_status_string(0) == b"ok"
    assert b"positive definite" in L.mcba_status_string(3)


def test_create_rejects_bad_precision():
    L = N.lib()
    o = N.Options()
    L.mcba_default_options(ctypes.byref(o))
    assert o.tau == 1e-5 and o.max_trials == 10
    o.precision = 7
    h = ctypes.c_void_p()
    assert L.mcba_create(ctypes.byref(o), ctypes.byref(h)) == 1


def test_graph_building_validation():
    s = Solver()
    L, h = s.L, s.h
    K = np.array([500, 500, 320, 240], np.float32)
    T = np.eye(4, dtype=np.float32).reshape(16)
    cid, kid, pid, eid = (ctypes.c_int32() for _ in range(4))
    fp = N.c_float_p
    assert L.mcba_add_camera(h, K.ctypes.data_as(fp), 0.0, T.ctypes.data_as(fp), ctypes.byref(cid)) == 0
    assert L.mcba_add_keyframe(h, T.ctypes.data_as(fp), 0, ctypes.byref(kid)) == 0
    X = np.array([0, 0, 5], np.float32)
    assert L.mcba_add_mappoint(h, X.ctypes.data_as(fp), 0, ctypes.byref(pid)) == 0
    assert L.mcba_add_edge_mono(h, 0, 0, 0, 320.0, 240.0, 1.0, 2.0, ctypes.byref(eid)) == 0
    assert eid.value == 0
    # unknown ids and non-finite values are rejected, nothing is added
    assert L.mcba_add_edge_mono(h, 5, 0, 0, 1.0, 1.0, 1.0, 2.0, None) == 1
    assert L.mcba_add_edge_mono(h, 0, 3, 0, 1.0, 1.0, 1.0, 2.0, None) == 1
    assert L.mcba_add_edge_mono(h, 0, 0, 9, 1.0, 1.0, 1.0, 2.0, None) == 1
    assert L.mcba_add_edge_mono(h, 0, 0, 0, float("nan"), 1.0, 1.0, 2.0, None) == 4
    bad = np.array([0, np.inf, 1], np.float32)
    assert L.mcba_add_mappoint(h, bad.ctypes.data_as(fp), 0, None) == 4
    n = ctypes.c_int32()
    L.mcba_edge_count(h, ctypes.byref(n))
    assert n.value == 1
    assert b"unknown" in L.mcba_last_error(h) or b"finite" in L.mcba_last_error(h)
    s.close()


def test_bulk_load_conversions_match_oracle():
    pr = synth.config(1)
    s = Solver().load(pr)
    qt, X = s.state()
    for k in range(pr.n_poses):
        np.testing.assert_array_equal(qt[k], oracle.mat44f_to_qt(pr.pose_Tcw[k]))
        T = s.keyframe(k)
        np.testing.assert_array_equal(T, oracle.qt_to_mat44f(qt[k]))
    np.testing.assert_array_equal(X, pr.point_Xw.astype(np.float64))
    lv = np.zeros(pr.n_edges, np.uint8)
    lv[::7] = 1
    s.set_levels(lv)
    np.testing.assert_array_equal(s.levels(), lv)
    s.close()


def test_bulk_load_rejects_out_of_range_edges():
    pr = synth.config(1)
    pr.edge_point = pr.edge_point.copy()
    pr.edge_point[3] = pr.n_points + 5
    s = Solver()
    with pytest.raises(N.MCBAError) as ei:
        s.load(pr)
    assert ei.value.status == 1
    s.close()


def test_optimize_without_device_reports_no_device():
    if N.device_count() > 0:
        pytest.skip("a CUDA device is present")
    s = Solver().load(synth.config(1))
    with pytest.raises(N.MCBAError) as ei:
        s.optimize(1)
    assert ei.value.status == 8
    s.close()


def test_empty_problem_is_reported_not_optimised():
    if N.device_count() == 0:
        pytest.skip("needs the device to reach the structure stage")
    pr = synth.config(1)
    pr.edge_level[:] = 1
    s = Solver().load(pr)
    st = s.optimize(3)
    assert st["ret"] == 2 and st["iterations"] == -1
    s.close()
