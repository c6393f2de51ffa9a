"""C-ABI boundary: exported symbols and host-side behaviour (no GPU needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

from state_estimation_with_cuda_gb300 import Estimator, SLEError, api, native

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for h in ("sle_api.h", "sle_ex.h"):
        with open(os.path.join(REPO, "include", h)) as fh:
            names += re.findall(r"SLE_CALL\s+(sle_\w+)\s*\(", fh.read())
    return names


def test_every_declared_symbol_is_exported():
    lib = native.sle_lib()
    names = declared_symbols()
    assert len(names) == 109  # 74 reference entry points + 35 additive sle_Ex*
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(native.SLE_SIGNATURES)


def test_version_and_real_size():
    lib = native.sle_lib()
    assert lib.sle_GetVersion() == b"0.20.0"
    assert lib.sle_ExRealSize() == 8
    assert lib.sle_GetDefaultConfigPath() == b"sle_engine.config"


def test_null_handle_errors():
    lib = native.sle_lib()
    assert lib.sle_Initialize(None) == api.ERROR_INVALID_HANDLE
    assert lib.sle_Solve(None, 0, None) == api.ERROR_INVALID_HANDLE
    assert lib.sle_Create(None) == api.ERROR_INVALID_ARGUMENT
    assert lib.sle_GetBusCount(None) == 0
    lib.sle_Destroy(None)  # NULL-safe


def test_model_building_error_codes():
    e = Estimator()
    e.add_bus("A", type=api.BUS_SLACK)
    e.add_bus("B")
    with pytest.raises(SLEError) as ex:
        e.add_bus("A")
    assert ex.value.code == api.ERROR_DUPLICATE_ID
    e.add_branch("AB", "A", "B", 0.01, 0.1)
    with pytest.raises(SLEError) as ex:  # reference maps every branch failure to ELEMENT_NOT_FOUND
        e.add_branch("AB", "A", "B", 0.01, 0.1)
    assert ex.value.code == api.ERROR_ELEMENT_NOT_FOUND
    with pytest.raises(SLEError) as ex:
        e.add_branch("AC", "A", "C", 0.01, 0.1)
    assert ex.value.code == api.ERROR_ELEMENT_NOT_FOUND
    e.add_measurement("V1", api.MEAS_V_MAG, "A", 0.004)
    with pytest.raises(SLEError) as ex:
        e.add_measurement("F1", api.MEAS_P_FLOW, "nope", 0.01)
    assert ex.value.code == api.ERROR_ELEMENT_NOT_FOUND
    assert e.counts() == (2, 1, 1)
    e.close()


def test_load_ieee14_counts_and_ids():
    e = Estimator()
    e.load_ieee14()
    assert e.counts() == (14, 20, 31)
    lib = e.lib
    assert lib.sle_GetMeasurementIdByIndex(e.h, 0) == b"V1"
    assert lib.sle_GetMeasurementIdByIndex(e.h, 30) == b"Q7_pseudo"
    assert lib.sle_GetTransformerTap(e.h, b"Xfmr4-7") == pytest.approx(0.978)
    e.close()


def test_meter_expansion_order():
    e = Estimator()
    e.add_bus("A", type=api.BUS_SLACK)
    e.add_bus("B")
    e.add_branch("L", "A", "B", 0.01, 0.1)
    mi = native.SLE_MeterInfo(b"MM1", 1, b"A", b"L", 0, 1.0, 1.0, 0.004, 0.01, 0.01)
    assert e.lib.sle_AddMeter(e.h, ctypes.byref(mi)) == 0
    ids = [e.lib.sle_GetMeasurementIdByIndex(e.h, i) for i in range(4)]
    assert ids == [b"MM1.V", b"MM1.kW", b"MM1.kVAR", b"MM1.A"]
    assert e.lib.sle_UpdateMeterReading(e.h, b"MM1", b"kW", 0.5) == 0
    v = ctypes.c_double()
    assert e.lib.sle_GetMeterReading(e.h, b"MM1", b"MW", ctypes.byref(v)) == 0 and v.value == 0.5
    assert e.lib.sle_GetMeterCount(e.h) == 1
    e.close()


def test_config_file_round_trip(tmp_path):
    lib = native.sle_lib()
    path = str(tmp_path / "sle.config").encode()
    c = native.SLE_Config()
    h = ctypes.c_void_p()
    assert lib.sle_Create(ctypes.byref(h)) == 0
    assert lib.sle_GetConfig(h, ctypes.byref(c)) == 0
    assert c.max_realtime_iterations == 5 and c.huber_gamma == 1.5 and c.bad_data_threshold == 3.0
    c.huber_gamma = 2.25
    c.max_precision_iterations = 33
    assert lib.sle_SaveConfigFile(path, ctypes.byref(c)) == 0
    c2 = native.SLE_Config()
    assert lib.sle_LoadConfigFile(path, ctypes.byref(c2)) == 0
    assert c2.huber_gamma == 2.25 and c2.max_precision_iterations == 33
    assert lib.sle_LoadConfigFile(b"/nonexistent/x.config", ctypes.byref(c2)) == api.ERROR_CONFIG_FILE
    lib.sle_Destroy(h)


def test_bulk_load_validates_indices():
    from state_estimation_with_cuda_gb300 import workloads

    g = workloads.make("grid14")
    e = Estimator()
    bad = g.br_from.copy()
    bad[0] = 99
    orig = g.br_from
    g.br_from = bad
    with pytest.raises(SLEError) as ex:
        e.load_network(g)
    assert ex.value.code == api.ERROR_ELEMENT_NOT_FOUND
    g.br_from = orig
    e.load_network(g)
    assert e.counts() == (g.n_bus, g.n_branch, g.n_meas)
    info = e.plan_info()  # host-only symbolic analysis
    assert info.n_state == 2 * g.n_bus - 1 and info.n_meas == g.n_meas
    e.close()


def test_bulk_load_default_names_and_edits():
    """A bulk-loaded model has no names until the first lookup, which gives
    every element its default name; adding and removing elements by name
    keep the names aligned with the element arrays."""
    from state_estimation_with_cuda_gb300 import workloads

    g = workloads.make("grid14")
    e = Estimator()
    e.load_network(g)
    lib = e.lib
    assert lib.sle_GetMeasurementIdByIndex(e.h, 0) == b"M0"
    assert lib.sle_GetMeasurementIdByIndex(e.h, g.n_meas - 1) == b"M%d" % (g.n_meas - 1)
    assert lib.sle_RemoveBranch(e.h, b"BR3") == 0
    nb, nbr, nm = e.counts()
    assert nbr == g.n_branch - 1
    assert lib.sle_GetMeasurementIdByIndex(e.h, nm - 1) is not None
    assert lib.sle_GetMeasurementIdByIndex(e.h, nm) is None
    assert lib.sle_RemoveBus(e.h, b"BUS5") == 0
    assert e.counts()[0] == nb - 1
    e.close()


def test_host_analysis_time_in_stats():
    """A host-only analysis (no device) counts itself and its host time in
    SLE_ExStats; nothing is uploaded or captured."""
    from state_estimation_with_cuda_gb300 import workloads

    g = workloads.make("grid14")
    e = Estimator()
    e.load_network(g)
    e.reset_stats()
    e.plan_info()
    s = e.stats()
    assert s.analyses == 1 and s.analysis_ms > 0
    assert s.uploads == 0 and s.upload_ms == 0 and s.capture_ms == 0
    e.close()


def test_removal_compacts_indices():
    e = Estimator()
    e.load_ieee14()
    e.lib.sle_RemoveBranch(e.h, b"Line1-2")
    nb, nbr, nm = e.counts()
    assert (nb, nbr) == (14, 19)
    assert nm == 29  # P1-2 and Q1-2 go with the branch
    assert e.lib.sle_GetMeasurementIdByIndex(e.h, 22) == b"P1-5"
    assert e.lib.sle_RemoveBus(e.h, b"Bus14") == 0
    assert e.counts()[0] == 13
    e.close()


def test_extension_options_validate_and_apply():
    """sle_ExSetOption keys (host side): every documented key is accepted with a
    valid value, out-of-range values are refused with INVALID_ARGUMENT, and an
    unknown key is refused."""
    e = Estimator()
    valid = {"exact_jacobian": 0, "gain_policy": 1, "ordering": 0, "use_double_precision": 0,
             "refine_steps": 1, "big_front_flops": 1e6, "dataflow": 1, "flow_small_f": 64, "warp_fronts": -1,
             "gain_accumulate": 64, "huber_stall": 1e-5, "spin_limit": 1 << 20, "hold_front": -1,
             "device_loop": 0, "tile_flow": 1, "eval_pair_rows": 0}
    for k, v in valid.items():
        e.set_option(k, v)
    for k, v in (("gain_accumulate", 16), ("huber_stall", 1.5), ("spin_limit", 0), ("eval_pair_rows", -1)):
        with pytest.raises(SLEError) as err:
            e.set_option(k, v)
        assert err.value.code == api.ERROR_INVALID_ARGUMENT
    with pytest.raises(SLEError):
        e.set_option("no_such_option", 1)
    e.close()


def test_stats_layout_matches_header():
    """SLE_ExStats as the header declares it: six stage arrays, the
    counters up to step_waits, then the four host phase times."""
    st = native.SLE_ExStats()
    names = [f[0] for f in st._fields_]
    assert names[:3] == ["launches", "ms", "calls"]
    assert names[-5:] == ["step_waits", "analysis_ms", "schedule_ms", "upload_ms", "capture_ms"]
    assert ctypes.sizeof(st) == 6 * 8 * 3 + 7 * 8 + 4 * 8
    e = Estimator()
    e.reset_stats()
    s = e.stats()
    assert s.step_waits == 0 and s.iterations == 0
    e.close()
