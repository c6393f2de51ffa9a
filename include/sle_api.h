/*
 * sle_api.h — C ABI of the GB300-native WLS state estimator.
 *
 * Drop-in replacement for the SLE Engine C API (reference include/sle_api.h):
 * the same function names, enumerations, structures and status codes, so an
 * application written against the reference links against libsle_gb300.so
 * unchanged.  Each declaration names the reference declaration it replaces.
 *
 * Precision: this library is the FP64 build of the ABI (the reference's
 * SLE_USE_DOUBLE configuration, reference include/sle_api.h:132-136), so
 * SLE_Real is double.  The header defines SLE_USE_DOUBLE itself; a caller
 * that needs to check at run time can compare sle_ExRealSize() (sle_ex.h)
 * with sizeof(SLE_Real).
 *
 * Threading: one handle is one engine and must not be used from two threads
 * at once; different handles may be used concurrently.  Error text from
 * sle_GetLastError is thread-local and valid until the next call on the same
 * thread.  Arrays passed in are copied before the call returns.
 */
#ifndef SLE_API_H
#define SLE_API_H

#include <stddef.h>
#include <stdint.h>

#ifndef SLE_USE_DOUBLE
#define SLE_USE_DOUBLE 1
#endif

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32) || defined(_WIN64)
#ifdef SLE_EXPORTS
#define SLE_API __declspec(dllexport)
#else
#define SLE_API __declspec(dllimport)
#endif
#define SLE_CALL __stdcall
#else
#define SLE_API __attribute__((visibility("default")))
#define SLE_CALL
#endif

#define SLE_VERSION_MAJOR 0
#define SLE_VERSION_MINOR 20
#define SLE_VERSION_PATCH 0
#define SLE_VERSION_STRING "0.20.0"

typedef struct SLE_EngineImpl* SLE_Handle;
typedef double SLE_Real;

/* reference include/sle_api.h:145-161 */
typedef enum SLE_StatusCode {
    SLE_OK = 0,
    SLE_ERROR_INVALID_HANDLE = -1,
    SLE_ERROR_NOT_INITIALIZED = -2,
    SLE_ERROR_CUDA_FAILURE = -3,
    SLE_ERROR_INVALID_ARGUMENT = -4,
    SLE_ERROR_MODEL_INCOMPLETE = -5,
    SLE_ERROR_NOT_OBSERVABLE = -6,
    SLE_ERROR_SINGULAR_MATRIX = -7,
    SLE_ERROR_DIVERGED = -8,
    SLE_ERROR_MAX_ITERATIONS = -9,
    SLE_ERROR_OUT_OF_MEMORY = -10,
    SLE_ERROR_ELEMENT_NOT_FOUND = -11,
    SLE_ERROR_DUPLICATE_ID = -12,
    SLE_ERROR_CONFIG_FILE = -13,
    SLE_ERROR_UNKNOWN = -99
} SLE_StatusCode;

/* reference include/sle_api.h:166-222 */
typedef enum SLE_BusType { SLE_BUS_PQ = 0, SLE_BUS_PV = 1, SLE_BUS_SLACK = 2 } SLE_BusType;
typedef enum SLE_SwitchStatus { SLE_SWITCH_OPEN = 0, SLE_SWITCH_CLOSED = 1 } SLE_SwitchStatus;
typedef enum SLE_MeasurementType {
    SLE_MEAS_V_MAG = 0,
    SLE_MEAS_V_ANGLE = 1,
    SLE_MEAS_P_INJECTION = 2,
    SLE_MEAS_Q_INJECTION = 3,
    SLE_MEAS_P_FLOW = 4,
    SLE_MEAS_Q_FLOW = 5,
    SLE_MEAS_I_MAG = 6,
    SLE_MEAS_P_PSEUDO = 7,
    SLE_MEAS_Q_PSEUDO = 8
} SLE_MeasurementType;
typedef enum SLE_BranchEnd { SLE_BRANCH_FROM = 0, SLE_BRANCH_TO = 1 } SLE_BranchEnd;
typedef enum SLE_EstimationMode { SLE_MODE_REALTIME = 0, SLE_MODE_PRECISION = 1 } SLE_EstimationMode;
typedef enum SLE_ConvergenceStatus {
    SLE_CONVERGED = 0,
    SLE_MAX_ITERATIONS = 1,
    SLE_DIVERGED = 2,
    SLE_SINGULAR = 3,
    SLE_NOT_OBSERVABLE = 4,
    SLE_IN_PROGRESS = 5
} SLE_ConvergenceStatus;

/* reference include/sle_api.h:230-237 */
typedef struct SLE_BusInfo {
    const char* id;
    SLE_Real base_kv;
    SLE_BusType type;
    SLE_Real v_setpoint;
    SLE_Real p_scheduled;
    SLE_Real q_scheduled;
} SLE_BusInfo;

/* reference include/sle_api.h:242-254 */
typedef struct SLE_BranchInfo {
    const char* id;
    const char* from_bus;
    const char* to_bus;
    SLE_Real resistance;
    SLE_Real reactance;
    SLE_Real susceptance;
    SLE_Real conductance;
    SLE_Real tap_ratio;
    SLE_Real phase_shift;
    int32_t is_transformer;
    const char* sd_id;
} SLE_BranchInfo;

/* reference include/sle_api.h:268-277 */
typedef struct SLE_MeasurementInfo {
    const char* id;
    SLE_MeasurementType type;
    const char* location;
    SLE_BranchEnd branch_end;
    SLE_Real sigma;
    SLE_Real pt_ratio;
    SLE_Real ct_ratio;
    int32_t is_pseudo;
} SLE_MeasurementInfo;

/* reference include/sle_api.h:282-287 */
typedef struct SLE_SwitchInfo {
    const char* id;
    const char* branch_id;
    SLE_SwitchStatus status;
} SLE_SwitchInfo;

/* reference include/sle_api.h:296-301 */
typedef enum SLE_MeterType {
    SLE_METER_VOLTMETER = 0,
    SLE_METER_MULTIMETER = 1,
    SLE_METER_AMMETER = 2,
    SLE_METER_WATTMETER = 3
} SLE_MeterType;

#define SLE_CHANNEL_VOLTAGE "V"
#define SLE_CHANNEL_VOLTAGE_KV "kV"
#define SLE_CHANNEL_CURRENT "A"
#define SLE_CHANNEL_CURRENT_KA "kA"
#define SLE_CHANNEL_POWER_KW "kW"
#define SLE_CHANNEL_POWER_MW "MW"
#define SLE_CHANNEL_REACTIVE_KVAR "kVAR"
#define SLE_CHANNEL_REACTIVE_MVAR "MVAR"
#define SLE_CHANNEL_ANGLE "deg"

/* reference include/sle_api.h:347-358 */
typedef struct SLE_MeterInfo {
    const char* id;
    SLE_MeterType type;
    const char* bus_id;
    const char* branch_id;
    SLE_BranchEnd branch_end;
    SLE_Real pt_ratio;
    SLE_Real ct_ratio;
    SLE_Real sigma_v;
    SLE_Real sigma_p;
    SLE_Real sigma_i;
} SLE_MeterInfo;

/* reference include/sle_api.h:363-367 */
typedef struct SLE_MeterReading {
    const char* meter_id;
    const char* channel;
    SLE_Real value;
} SLE_MeterReading;

/* reference include/sle_api.h:370-379 */
typedef struct SLE_Result {
    SLE_ConvergenceStatus status;
    int32_t iterations;
    SLE_Real max_mismatch;
    SLE_Real objective;
    SLE_Real computation_time_ms;
    SLE_Real largest_residual;
    int32_t largest_residual_idx;
    int32_t bad_data_count;
} SLE_Result;

/* reference include/sle_api.h:386-419.  use_double_precision selects the
 * numeric pipeline: 1 = plain FP64 throughout, 0 = mixed precision (FP32
 * Jacobian, gain and factor with FP64 residual, refinement and state). */
typedef struct SLE_Config {
    int32_t device_id;
    size_t max_buses;
    size_t max_branches;
    size_t max_measurements;
    size_t max_switching_devices;
    int32_t enable_robust;
    SLE_Real huber_gamma;
    SLE_Real convergence_tolerance;
    int32_t max_realtime_iterations;
    int32_t max_precision_iterations;
    SLE_Real realtime_time_limit_ms;
    int32_t use_flat_start_default;
    int32_t enable_profiling;
    int32_t use_cuda_graphs;
    int32_t block_size_standard;
    int32_t block_size_reduction;
    int32_t use_double_precision;
    SLE_Real voltage_min_pu;
    SLE_Real voltage_max_pu;
    SLE_Real bad_data_threshold;
    int32_t auto_bad_data_rejection;
} SLE_Config;

/* reference include/sle_api.h:424-432 */
typedef struct SLE_SolverConfig {
    SLE_EstimationMode mode;
    int32_t max_iterations;
    SLE_Real tolerance;
    SLE_Real huber_gamma;
    int32_t use_robust;
    int32_t use_flat_start;
    SLE_Real time_limit_ms;
} SLE_SolverConfig;

/* reference include/sle_api.h:953-957 */
typedef struct SLE_MeasurementUpdate {
    const char* meas_id;
    SLE_Real value;
} SLE_MeasurementUpdate;

/* reference include/sle_api.h:1011-1025 */
typedef struct SLE_MeasurementDetails {
    const char* id;
    SLE_MeasurementType type;
    const char* location_id;
    SLE_BranchEnd branch_end;
    SLE_Real sigma;
    SLE_Real pt_ratio;
    SLE_Real ct_ratio;
    int32_t is_pseudo;
    int32_t internal_index;
    SLE_Real current_value;
    SLE_Real estimated_value;
    SLE_Real residual;
    int32_t is_active;
} SLE_MeasurementDetails;

/* ---- lifecycle (reference include/sle_api.h:447-487) ---- */
SLE_API SLE_StatusCode SLE_CALL sle_Create(SLE_Handle* handle);
SLE_API SLE_StatusCode SLE_CALL sle_CreateWithConfig(SLE_Handle* handle, const SLE_Config* config);
SLE_API SLE_StatusCode SLE_CALL sle_CreateFromConfigFile(SLE_Handle* handle, const char* config_path);
SLE_API SLE_StatusCode SLE_CALL sle_Initialize(SLE_Handle handle);
SLE_API void SLE_CALL sle_Destroy(SLE_Handle handle);

/* ---- configuration (reference include/sle_api.h:503-584) ---- */
SLE_API SLE_StatusCode SLE_CALL sle_LoadConfigFile(const char* config_path, SLE_Config* config);
SLE_API SLE_StatusCode SLE_CALL sle_SaveConfigFile(const char* config_path, const SLE_Config* config);
SLE_API SLE_StatusCode SLE_CALL sle_ReloadConfig(SLE_Handle handle);
SLE_API SLE_StatusCode SLE_CALL sle_ReloadConfigFromFile(SLE_Handle handle, const char* config_path);
SLE_API const char* SLE_CALL sle_GetDefaultConfigPath(void);
SLE_API const char* SLE_CALL sle_GetConfigPath(SLE_Handle handle);
SLE_API SLE_StatusCode SLE_CALL sle_EnsureConfigFile(const char* config_path);
SLE_API SLE_StatusCode SLE_CALL sle_GetConfig(SLE_Handle handle, SLE_Config* config);
SLE_API SLE_StatusCode SLE_CALL sle_SetConfig(SLE_Handle handle, const SLE_Config* config);

/* ---- errors / device (reference include/sle_api.h:597-605) ---- */
SLE_API const char* SLE_CALL sle_GetLastError(SLE_Handle handle);
SLE_API const char* SLE_CALL sle_GetDeviceInfo(SLE_Handle handle);

/* ---- model building (reference include/sle_api.h:610-749) ---- */
SLE_API SLE_StatusCode SLE_CALL sle_AddBus(SLE_Handle handle, const SLE_BusInfo* info);
SLE_API SLE_StatusCode SLE_CALL sle_AddBuses(SLE_Handle handle, const SLE_BusInfo* buses, int32_t count);
SLE_API SLE_StatusCode SLE_CALL sle_AddBranch(SLE_Handle handle, const SLE_BranchInfo* info);
SLE_API SLE_StatusCode SLE_CALL sle_AddBranches(SLE_Handle handle, const SLE_BranchInfo* branches, int32_t count);
SLE_API SLE_StatusCode SLE_CALL sle_AddMeasurement(SLE_Handle handle, const SLE_MeasurementInfo* info);
SLE_API SLE_StatusCode SLE_CALL sle_AddMeasurements(SLE_Handle handle, const SLE_MeasurementInfo* meas, int32_t count);
SLE_API SLE_StatusCode SLE_CALL sle_AddSwitch(SLE_Handle handle, const SLE_SwitchInfo* info);
SLE_API SLE_StatusCode SLE_CALL sle_RemoveBus(SLE_Handle handle, const char* bus_id);
SLE_API SLE_StatusCode SLE_CALL sle_RemoveBranch(SLE_Handle handle, const char* branch_id);
SLE_API SLE_StatusCode SLE_CALL sle_UpdateBranch(SLE_Handle handle, const SLE_BranchInfo* info);
SLE_API SLE_StatusCode SLE_CALL sle_SetTransformerTap(SLE_Handle handle, const char* branch_id, SLE_Real tap_ratio);
SLE_API SLE_StatusCode SLE_CALL sle_SetTransformerPhaseShift(SLE_Handle handle, const char* branch_id,
                                                             SLE_Real phase_shift);
SLE_API SLE_StatusCode SLE_CALL sle_SetBranchImpedance(SLE_Handle handle, const char* branch_id, SLE_Real r,
                                                       SLE_Real x, SLE_Real b, SLE_Real g);
SLE_API SLE_Real SLE_CALL sle_GetTransformerTap(SLE_Handle handle, const char* branch_id);
SLE_API SLE_Real SLE_CALL sle_GetTransformerPhaseShift(SLE_Handle handle, const char* branch_id);

/* ---- meters (reference include/sle_api.h:828-910) ---- */
SLE_API SLE_StatusCode SLE_CALL sle_AddMeter(SLE_Handle handle, const SLE_MeterInfo* info);
SLE_API SLE_StatusCode SLE_CALL sle_UpdateMeterReading(SLE_Handle handle, const char* meter_id, const char* channel,
                                                       SLE_Real value);
SLE_API SLE_StatusCode SLE_CALL sle_UpdateMeterReadings(SLE_Handle handle, const SLE_MeterReading* readings,
                                                        int32_t count, int32_t sync_to_device);
SLE_API SLE_StatusCode SLE_CALL sle_GetMeterReading(SLE_Handle handle, const char* meter_id, const char* channel,
                                                    SLE_Real* value);
SLE_API SLE_StatusCode SLE_CALL sle_GetMeterEstimate(SLE_Handle handle, const char* meter_id, const char* channel,
                                                     SLE_Real* value);
SLE_API SLE_StatusCode SLE_CALL sle_GetMeterResidual(SLE_Handle handle, const char* meter_id, const char* channel,
                                                     SLE_Real* residual);

/* ---- device data (reference include/sle_api.h:935-1052) ---- */
SLE_API SLE_StatusCode SLE_CALL sle_UploadModel(SLE_Handle handle);
SLE_API SLE_StatusCode SLE_CALL sle_UpdateTelemetry(SLE_Handle handle, const SLE_Real* values, int32_t count);
SLE_API SLE_StatusCode SLE_CALL sle_UpdateMeasurement(SLE_Handle handle, const char* meas_id, SLE_Real value);
SLE_API SLE_StatusCode SLE_CALL sle_UpdateMeasurementBatch(SLE_Handle handle, const SLE_MeasurementUpdate* updates,
                                                           int32_t count, int32_t sync_to_device);
SLE_API SLE_StatusCode SLE_CALL sle_SyncMeasurementsToDevice(SLE_Handle handle);
SLE_API SLE_StatusCode SLE_CALL sle_GetMeasurementDetails(SLE_Handle handle, const char* meas_id,
                                                          SLE_MeasurementDetails* details);
SLE_API const char* SLE_CALL sle_GetMeasurementIdByIndex(SLE_Handle handle, int32_t index);

/* ---- switches (reference include/sle_api.h:1063-1084) ---- */
SLE_API SLE_StatusCode SLE_CALL sle_SetSwitchStatus(SLE_Handle handle, const char* sd_id, SLE_SwitchStatus status);
SLE_API SLE_SwitchStatus SLE_CALL sle_GetSwitchStatus(SLE_Handle handle, const char* sd_id);
SLE_API SLE_StatusCode SLE_CALL sle_ApplySwitchChanges(SLE_Handle handle);

/* ---- estimation (reference include/sle_api.h:1102-1135) ---- */
SLE_API SLE_StatusCode SLE_CALL sle_Solve(SLE_Handle handle, SLE_EstimationMode mode, SLE_Result* result);
SLE_API SLE_StatusCode SLE_CALL sle_SolveWithConfig(SLE_Handle handle, const SLE_SolverConfig* config,
                                                    SLE_Result* result);
SLE_API SLE_StatusCode SLE_CALL sle_CheckObservability(SLE_Handle handle, int32_t* is_observable,
                                                       int32_t* island_count);
SLE_API SLE_StatusCode SLE_CALL sle_ApplyFlatStart(SLE_Handle handle);

/* ---- results (reference include/sle_api.h:1153-1311) ---- */
SLE_API SLE_StatusCode SLE_CALL sle_GetVoltageMagnitudes(SLE_Handle handle, SLE_Real* values, int32_t count);
SLE_API SLE_StatusCode SLE_CALL sle_GetVoltageAngles(SLE_Handle handle, SLE_Real* values, int32_t count);
SLE_API SLE_Real SLE_CALL sle_GetBusVoltage(SLE_Handle handle, const char* bus_id);
SLE_API SLE_Real SLE_CALL sle_GetBusAngle(SLE_Handle handle, const char* bus_id);
SLE_API SLE_StatusCode SLE_CALL sle_GetPowerInjections(SLE_Handle handle, SLE_Real* p_values, SLE_Real* q_values,
                                                       int32_t count);
SLE_API SLE_StatusCode SLE_CALL sle_GetBranchFlows(SLE_Handle handle, SLE_Real* p_from, SLE_Real* q_from,
                                                   SLE_Real* p_to, SLE_Real* q_to, int32_t count);
SLE_API SLE_Real SLE_CALL sle_GetBranchP(SLE_Handle handle, const char* branch_id, SLE_BranchEnd end);
SLE_API SLE_Real SLE_CALL sle_GetBranchQ(SLE_Handle handle, const char* branch_id, SLE_BranchEnd end);
SLE_API SLE_StatusCode SLE_CALL sle_GetBusResiduals(SLE_Handle handle, const char* bus_id, SLE_Real* v_residual,
                                                    SLE_Real* p_residual, SLE_Real* q_residual, int32_t* count);
SLE_API SLE_StatusCode SLE_CALL sle_GetBranchResiduals(SLE_Handle handle, const char* branch_id, SLE_BranchEnd end,
                                                       SLE_Real* p_residual, SLE_Real* q_residual,
                                                       SLE_Real* i_residual, int32_t* count);
SLE_API SLE_StatusCode SLE_CALL sle_GetResiduals(SLE_Handle handle, SLE_Real* values, int32_t count);
SLE_API SLE_Real SLE_CALL sle_GetObjective(SLE_Handle handle);
SLE_API SLE_StatusCode SLE_CALL sle_IdentifyBadData(SLE_Handle handle, SLE_Real threshold, int32_t* indices,
                                                    int32_t max_count, int32_t* actual_count);

/* ---- model information (reference include/sle_api.h:1320-1351) ---- */
SLE_API int32_t SLE_CALL sle_GetBusCount(SLE_Handle handle);
SLE_API int32_t SLE_CALL sle_GetBranchCount(SLE_Handle handle);
SLE_API int32_t SLE_CALL sle_GetMeasurementCount(SLE_Handle handle);
SLE_API int32_t SLE_CALL sle_GetMeterCount(SLE_Handle handle);
SLE_API size_t SLE_CALL sle_GetGPUMemoryUsage(SLE_Handle handle);
SLE_API SLE_Real SLE_CALL sle_GetLastSolveTime(SLE_Handle handle);

/* ---- test case / system (reference include/sle_api.h:1366-1390) ---- */
SLE_API SLE_StatusCode SLE_CALL sle_LoadIEEE14Bus(SLE_Handle handle);
SLE_API const char* SLE_CALL sle_GetVersion(void);
SLE_API int32_t SLE_CALL sle_GetCUDAVersion(void);
SLE_API int32_t SLE_CALL sle_IsGPUAvailable(void);

#ifdef __cplusplus
}
#endif
#endif /* SLE_API_H */
