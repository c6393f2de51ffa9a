"""ctypes loading of the in-tree native libraries.

The product path is libsle_gb300.so (C ABI + sm_103a kernels); there is no
Python or CPU fallback: importing a missing library raises.
"""
import ctypes
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(PKG, "lib")

_libs = {}


class NativeLibraryMissing(RuntimeError):
    pass


def _load(name):
    if name in _libs:
        return _libs[name]
    path = os.path.join(LIB_DIR, name)
    if not os.path.exists(path):
        raise NativeLibraryMissing("%s is not built; run `python -c \"import __graft_entry__ as g; g.build()\"`" % path)
    lib = ctypes.CDLL(path)
    _libs[name] = lib
    return lib


c_int32_p = ctypes.POINTER(ctypes.c_int32)
c_int64_p = ctypes.POINTER(ctypes.c_int64)
c_double_p = ctypes.POINTER(ctypes.c_double)


class SLE_BusInfo(ctypes.Structure):
    _fields_ = [("id", ctypes.c_char_p), ("base_kv", ctypes.c_double), ("type", ctypes.c_int),
                ("v_setpoint", ctypes.c_double), ("p_scheduled", ctypes.c_double), ("q_scheduled", ctypes.c_double)]


class SLE_BranchInfo(ctypes.Structure):
    _fields_ = [("id", ctypes.c_char_p), ("from_bus", ctypes.c_char_p), ("to_bus", ctypes.c_char_p),
                ("resistance", ctypes.c_double), ("reactance", ctypes.c_double), ("susceptance", ctypes.c_double),
                ("conductance", ctypes.c_double), ("tap_ratio", ctypes.c_double), ("phase_shift", ctypes.c_double),
                ("is_transformer", ctypes.c_int32), ("sd_id", ctypes.c_char_p)]


class SLE_MeasurementInfo(ctypes.Structure):
    _fields_ = [("id", ctypes.c_char_p), ("type", ctypes.c_int), ("location", ctypes.c_char_p),
                ("branch_end", ctypes.c_int), ("sigma", ctypes.c_double), ("pt_ratio", ctypes.c_double),
                ("ct_ratio", ctypes.c_double), ("is_pseudo", ctypes.c_int32)]


class SLE_SwitchInfo(ctypes.Structure):
    _fields_ = [("id", ctypes.c_char_p), ("branch_id", ctypes.c_char_p), ("status", ctypes.c_int)]


class SLE_MeterInfo(ctypes.Structure):
    _fields_ = [("id", ctypes.c_char_p), ("type", ctypes.c_int), ("bus_id", ctypes.c_char_p),
                ("branch_id", ctypes.c_char_p), ("branch_end", ctypes.c_int), ("pt_ratio", ctypes.c_double),
                ("ct_ratio", ctypes.c_double), ("sigma_v", ctypes.c_double), ("sigma_p", ctypes.c_double),
                ("sigma_i", ctypes.c_double)]


class SLE_MeterReading(ctypes.Structure):
    _fields_ = [("meter_id", ctypes.c_char_p), ("channel", ctypes.c_char_p), ("value", ctypes.c_double)]


class SLE_Result(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("iterations", ctypes.c_int32), ("max_mismatch", ctypes.c_double),
                ("objective", ctypes.c_double), ("computation_time_ms", ctypes.c_double),
                ("largest_residual", ctypes.c_double), ("largest_residual_idx", ctypes.c_int32),
                ("bad_data_count", ctypes.c_int32)]


class SLE_ExGridResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("iterations", ctypes.c_int32), ("max_mismatch", ctypes.c_double),
                ("objective", ctypes.c_double)]


class SLE_ExServerConfig(ctypes.Structure):
    _fields_ = [("use_double_precision", ctypes.c_int32), ("max_iterations", ctypes.c_int32),
                ("tolerance", ctypes.c_double), ("robust", ctypes.c_int32), ("huber_gamma", ctypes.c_double),
                ("bucket_bus", ctypes.c_int32 * 4), ("own_unit_bus", ctypes.c_int32), ("device_id", ctypes.c_int32),
                ("memory_budget", ctypes.c_size_t)]


class SLE_ExServeResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("iterations", ctypes.c_int32), ("max_mismatch", ctypes.c_double),
                ("objective", ctypes.c_double), ("admitted", ctypes.c_int32), ("batch_size", ctypes.c_int32),
                ("t_submit_ns", ctypes.c_int64), ("t_start_ns", ctypes.c_int64), ("t_done_ns", ctypes.c_int64)]


class SLE_ExServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_int64), ("completed", ctypes.c_int64), ("rejected", ctypes.c_int64),
                ("passes", ctypes.c_int64), ("grid_solves", ctypes.c_int64), ("units", ctypes.c_int32),
                ("admitted_units", ctypes.c_int32), ("grids", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("device_bytes", ctypes.c_size_t), ("budget_bytes", ctypes.c_size_t),
                ("admissions", ctypes.c_int64), ("evictions", ctypes.c_int64), ("resident_units", ctypes.c_int32),
                ("pad2", ctypes.c_int32)]


class SLE_Config(ctypes.Structure):
    _fields_ = [("device_id", ctypes.c_int32), ("max_buses", ctypes.c_size_t), ("max_branches", ctypes.c_size_t),
                ("max_measurements", ctypes.c_size_t), ("max_switching_devices", ctypes.c_size_t),
                ("enable_robust", ctypes.c_int32), ("huber_gamma", ctypes.c_double),
                ("convergence_tolerance", ctypes.c_double), ("max_realtime_iterations", ctypes.c_int32),
                ("max_precision_iterations", ctypes.c_int32), ("realtime_time_limit_ms", ctypes.c_double),
                ("use_flat_start_default", ctypes.c_int32), ("enable_profiling", ctypes.c_int32),
                ("use_cuda_graphs", ctypes.c_int32), ("block_size_standard", ctypes.c_int32),
                ("block_size_reduction", ctypes.c_int32), ("use_double_precision", ctypes.c_int32),
                ("voltage_min_pu", ctypes.c_double), ("voltage_max_pu", ctypes.c_double),
                ("bad_data_threshold", ctypes.c_double), ("auto_bad_data_rejection", ctypes.c_int32)]


class SLE_SolverConfig(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int), ("max_iterations", ctypes.c_int32), ("tolerance", ctypes.c_double),
                ("huber_gamma", ctypes.c_double), ("use_robust", ctypes.c_int32), ("use_flat_start", ctypes.c_int32),
                ("time_limit_ms", ctypes.c_double)]


class SLE_MeasurementUpdate(ctypes.Structure):
    _fields_ = [("meas_id", ctypes.c_char_p), ("value", ctypes.c_double)]


class SLE_MeasurementDetails(ctypes.Structure):
    _fields_ = [("id", ctypes.c_char_p), ("type", ctypes.c_int), ("location_id", ctypes.c_char_p),
                ("branch_end", ctypes.c_int), ("sigma", ctypes.c_double), ("pt_ratio", ctypes.c_double),
                ("ct_ratio", ctypes.c_double), ("is_pseudo", ctypes.c_int32), ("internal_index", ctypes.c_int32),
                ("current_value", ctypes.c_double), ("estimated_value", ctypes.c_double),
                ("residual", ctypes.c_double), ("is_active", ctypes.c_int32)]


class SLE_ExPlanInfo(ctypes.Structure):
    _fields_ = [("n_bus", ctypes.c_int32), ("n_state", ctypes.c_int32), ("n_meas", ctypes.c_int32),
                ("nnz_ybus", ctypes.c_int32), ("nnz_h", ctypes.c_int64), ("n_super", ctypes.c_int32),
                ("n_levels", ctypes.c_int32), ("max_front", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("nnz_l", ctypes.c_int64), ("lx_size", ctypes.c_int64), ("u_size", ctypes.c_int64),
                ("n_gain_targets", ctypes.c_int64), ("n_gain_pairs", ctypes.c_int64),
                ("factor_flops", ctypes.c_double), ("device_bytes", ctypes.c_size_t)]


class SLE_ExScheduleInfo(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in (
        "n_warp", "n_phase_a", "n_phase_b", "n_sync", "warp_ready", "a_ready", "b_ready", "up_ready", "down_n",
        "down_warp_n", "sync_levels", "panel_steps", "by_depth", "tile_tasks")] + [
        ("launches_by_height", ctypes.c_int64), ("launches_by_depth", ctypes.c_int64)]


class SLE_ExStats(ctypes.Structure):
    _fields_ = [("launches", ctypes.c_int64 * 6), ("ms", ctypes.c_double * 6), ("calls", ctypes.c_int64 * 6),
                ("iterations", ctypes.c_int64), ("solves", ctypes.c_int64), ("total_launches", ctypes.c_int64),
                ("analyses", ctypes.c_int64), ("uploads", ctypes.c_int64), ("branch_edits", ctypes.c_int64),
                ("step_waits", ctypes.c_int64), ("analysis_ms", ctypes.c_double), ("schedule_ms", ctypes.c_double),
                ("upload_ms", ctypes.c_double), ("capture_ms", ctypes.c_double)]


H = ctypes.c_void_p
I = ctypes.c_int32
D = ctypes.c_double
S = ctypes.c_char_p
P = ctypes.POINTER

# name -> (restype, argtypes)
SLE_SIGNATURES = {
    "sle_Create": (I, [P(H)]),
    "sle_CreateWithConfig": (I, [P(H), P(SLE_Config)]),
    "sle_CreateFromConfigFile": (I, [P(H), S]),
    "sle_Initialize": (I, [H]),
    "sle_Destroy": (None, [H]),
    "sle_LoadConfigFile": (I, [S, P(SLE_Config)]),
    "sle_SaveConfigFile": (I, [S, P(SLE_Config)]),
    "sle_ReloadConfig": (I, [H]),
    "sle_ReloadConfigFromFile": (I, [H, S]),
    "sle_GetDefaultConfigPath": (S, []),
    "sle_GetConfigPath": (S, [H]),
    "sle_EnsureConfigFile": (I, [S]),
    "sle_GetConfig": (I, [H, P(SLE_Config)]),
    "sle_SetConfig": (I, [H, P(SLE_Config)]),
    "sle_GetLastError": (S, [H]),
    "sle_GetDeviceInfo": (S, [H]),
    "sle_AddBus": (I, [H, P(SLE_BusInfo)]),
    "sle_AddBuses": (I, [H, P(SLE_BusInfo), I]),
    "sle_AddBranch": (I, [H, P(SLE_BranchInfo)]),
    "sle_AddBranches": (I, [H, P(SLE_BranchInfo), I]),
    "sle_AddMeasurement": (I, [H, P(SLE_MeasurementInfo)]),
    "sle_AddMeasurements": (I, [H, P(SLE_MeasurementInfo), I]),
    "sle_AddSwitch": (I, [H, P(SLE_SwitchInfo)]),
    "sle_RemoveBus": (I, [H, S]),
    "sle_RemoveBranch": (I, [H, S]),
    "sle_UpdateBranch": (I, [H, P(SLE_BranchInfo)]),
    "sle_SetTransformerTap": (I, [H, S, D]),
    "sle_SetTransformerPhaseShift": (I, [H, S, D]),
    "sle_SetBranchImpedance": (I, [H, S, D, D, D, D]),
    "sle_GetTransformerTap": (D, [H, S]),
    "sle_GetTransformerPhaseShift": (D, [H, S]),
    "sle_AddMeter": (I, [H, P(SLE_MeterInfo)]),
    "sle_UpdateMeterReading": (I, [H, S, S, D]),
    "sle_UpdateMeterReadings": (I, [H, P(SLE_MeterReading), I, I]),
    "sle_GetMeterReading": (I, [H, S, S, P(D)]),
    "sle_GetMeterEstimate": (I, [H, S, S, P(D)]),
    "sle_GetMeterResidual": (I, [H, S, S, P(D)]),
    "sle_UploadModel": (I, [H]),
    "sle_UpdateTelemetry": (I, [H, P(D), I]),
    "sle_UpdateMeasurement": (I, [H, S, D]),
    "sle_UpdateMeasurementBatch": (I, [H, P(SLE_MeasurementUpdate), I, I]),
    "sle_SyncMeasurementsToDevice": (I, [H]),
    "sle_GetMeasurementDetails": (I, [H, S, P(SLE_MeasurementDetails)]),
    "sle_GetMeasurementIdByIndex": (S, [H, I]),
    "sle_SetSwitchStatus": (I, [H, S, I]),
    "sle_GetSwitchStatus": (I, [H, S]),
    "sle_ApplySwitchChanges": (I, [H]),
    "sle_Solve": (I, [H, I, P(SLE_Result)]),
    "sle_SolveWithConfig": (I, [H, P(SLE_SolverConfig), P(SLE_Result)]),
    "sle_CheckObservability": (I, [H, P(I), P(I)]),
    "sle_ApplyFlatStart": (I, [H]),
    "sle_GetVoltageMagnitudes": (I, [H, P(D), I]),
    "sle_GetVoltageAngles": (I, [H, P(D), I]),
    "sle_GetBusVoltage": (D, [H, S]),
    "sle_GetBusAngle": (D, [H, S]),
    "sle_GetPowerInjections": (I, [H, P(D), P(D), I]),
    "sle_GetBranchFlows": (I, [H, P(D), P(D), P(D), P(D), I]),
    "sle_GetBranchP": (D, [H, S, I]),
    "sle_GetBranchQ": (D, [H, S, I]),
    "sle_GetBusResiduals": (I, [H, S, P(D), P(D), P(D), P(I)]),
    "sle_GetBranchResiduals": (I, [H, S, I, P(D), P(D), P(D), P(I)]),
    "sle_GetResiduals": (I, [H, P(D), I]),
    "sle_GetObjective": (D, [H]),
    "sle_IdentifyBadData": (I, [H, D, P(I), I, P(I)]),
    "sle_GetBusCount": (I, [H]),
    "sle_GetBranchCount": (I, [H]),
    "sle_GetMeasurementCount": (I, [H]),
    "sle_GetMeterCount": (I, [H]),
    "sle_GetGPUMemoryUsage": (ctypes.c_size_t, [H]),
    "sle_GetLastSolveTime": (D, [H]),
    "sle_LoadIEEE14Bus": (I, [H]),
    "sle_GetVersion": (S, []),
    "sle_GetCUDAVersion": (I, []),
    "sle_IsGPUAvailable": (I, []),
    # additive extensions (sle_ex.h)
    "sle_ExRealSize": (I, []),
    "sle_ExLoadNetwork": (I, [H, I, P(I), P(D), I, P(I), P(I), P(D), P(D), P(D), P(D), P(D), P(I), I, P(I), P(I),
                              P(I), P(D), P(D)]),
    "sle_ExSetOption": (I, [H, S, D]),
    "sle_ExGetPlanInfo": (I, [H, P(SLE_ExPlanInfo)]),
    "sle_ExGetScheduleInfo": (I, [H, P(SLE_ExScheduleInfo)]),
    "sle_ExGetYbus": (I, [H, P(I), P(I), P(D), P(D)]),
    "sle_ExEvaluateAt": (I, [H, P(D), P(D), I]),
    "sle_ExGetJacobian": (I, [H, P(I), P(I), P(D), P(D), P(D)]),
    "sle_ExGetGain": (I, [H, P(I), P(I), P(D)]),
    "sle_ExFactorSolve": (I, [H, P(D), P(D)]),
    "sle_ExFactorSolveNoAlloc": (I, [H, P(D), P(D)]),
    "sle_ExGetSymbolic": (I, [H, P(I), P(I), P(I), P(I), P(ctypes.c_int64), P(I)]),
    "sle_ExStageTelemetry": (I, [H, P(D), I, I]),
    "sle_ExUseTelemetry": (I, [H, I]),
    "sle_ExFlushL2": (I, [H, ctypes.c_size_t]),
    "sle_ExTimer": (I, [H, I, P(D)]),
    "sle_ExGetStats": (I, [H, P(SLE_ExStats)]),
    "sle_ExResetStats": (I, [H]),
    "sle_ExBatchAddGrid": (I, [H, I, P(I), P(D), I, P(I), P(I), P(D), P(D), P(D), P(D), P(D), P(I), I, P(I), P(I),
                               P(I), P(D), P(D), P(I)]),
    "sle_ExBatchGridCount": (I, [H]),
    "sle_ExBatchUpdateTelemetry": (I, [H, I, P(D), I]),
    "sle_ExBatchSolve": (I, [H, I, P(I), P(ctypes.c_uint8), I, D, I, D, P(SLE_ExGridResult)]),
    "sle_ExBatchGetState": (I, [H, I, P(D), P(D)]),
    "sle_ExBatchSetBranchStatus": (I, [H, I, I, I]),
    "sle_ExServerDefaultConfig": (None, [P(SLE_ExServerConfig)]),
    "sle_ExServerCreate": (I, [P(ctypes.c_void_p), P(SLE_ExServerConfig)]),
    "sle_ExServerDestroy": (None, [ctypes.c_void_p]),
    "sle_ExServerAddGrid": (I, [ctypes.c_void_p, I, P(I), P(D), I, P(I), P(I), P(D), P(D), P(D), P(D), P(D), P(I), I,
                                P(I), P(I), P(I), P(D), P(D), P(I)]),
    "sle_ExServerStart": (I, [ctypes.c_void_p]),
    "sle_ExServerSubmit": (I, [ctypes.c_void_p, I, P(D), I, I, I, P(ctypes.c_int64)]),
    "sle_ExServerSubmitEx": (I, [ctypes.c_void_p, I, P(D), I, I, I, P(D), P(D), P(ctypes.c_int64)]),
    "sle_ExServerWait": (I, [ctypes.c_void_p, ctypes.c_int64, D, P(SLE_ExServeResult)]),
    "sle_ExServerGetState": (I, [ctypes.c_void_p, I, P(D), P(D)]),
    "sle_ExServerGetStats": (I, [ctypes.c_void_p, P(SLE_ExServerStats)]),
    "sle_ExServerLastError": (S, [ctypes.c_void_p]),
}


def sle_lib():
    lib = _load("libsle_gb300.so")
    if not getattr(lib, "_sle_typed", False):
        for name, (res, args) in SLE_SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        lib._sle_typed = True
    return lib


class SEGenParams(ctypes.Structure):
    _fields_ = [("n_bus", ctypes.c_int32), ("n_branch", ctypes.c_int32), ("seed", ctypes.c_uint64),
                ("frac_vmag", ctypes.c_double), ("frac_inj", ctypes.c_double), ("frac_flow", ctypes.c_double),
                ("n_vmag", ctypes.c_int32), ("n_inj", ctypes.c_int32), ("n_flow", ctypes.c_int32),
                ("n_tap", ctypes.c_int32), ("sigma_v", ctypes.c_double), ("sigma_inj", ctypes.c_double),
                ("sigma_flow", ctypes.c_double), ("gross_frac", ctypes.c_double), ("sigma_pseudo", ctypes.c_double)]


def segen_lib():
    lib = _load("libsegen.so")
    if not getattr(lib, "_typed", False):
        lib.segen_default_params.argtypes = [P(SEGenParams), I, I, ctypes.c_uint64]
        lib.segen_create.restype = ctypes.c_void_p
        lib.segen_create.argtypes = [P(SEGenParams)]
        lib.segen_destroy.argtypes = [ctypes.c_void_p]
        for name in ("segen_n_bus", "segen_n_branch", "segen_n_meas", "segen_slack"):
            getattr(lib, name).restype = I
            getattr(lib, name).argtypes = [ctypes.c_void_p]
        for name in ("segen_bus_type", "segen_br_from", "segen_br_to", "segen_br_status", "segen_meas_type",
                     "segen_meas_loc", "segen_meas_end", "segen_meas_gross"):
            getattr(lib, name).restype = P(I)
            getattr(lib, name).argtypes = [ctypes.c_void_p]
        for name in ("segen_v_setpoint", "segen_v_true", "segen_theta_true", "segen_br_r", "segen_br_x",
                     "segen_br_b", "segen_br_tap", "segen_br_shift", "segen_meas_sigma", "segen_meas_z",
                     "segen_meas_htrue"):
            getattr(lib, name).restype = P(D)
            getattr(lib, name).argtypes = [ctypes.c_void_p]
        lib.segen_renoise.restype = I
        lib.segen_renoise.argtypes = [ctypes.c_void_p, I, D, P(D)]
        lib.segen_set_status.argtypes = [ctypes.c_void_p, I, I]
        lib.segen_pick_nonbridge.restype = I
        lib.segen_pick_nonbridge.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        lib.segen_draw_loguniform.restype = I
        lib.segen_draw_loguniform.argtypes = [ctypes.c_uint64, I, I, I]
        lib.segen_draw_zipf.restype = I
        lib.segen_draw_zipf.argtypes = [ctypes.c_uint64, I, D, I, I]
        lib._typed = True
    return lib
