// C ABI: the reference's sle_* entry points (reference src/sle_api.cu) backed
// by the GB300 engine, plus the additive sle_Ex* entry points of sle_ex.h.
#define SLE_EXPORTS 1
#include "../../../include/sle_api.h"
#include "../../../include/sle_ex.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

#include "../engine/engine.h"
#include "../serve/server.h"

using sle_gb300::Engine;
using sle_gb300::EngineConfig;

namespace {

thread_local std::string g_last_error;  // thread-local, not per handle (sle_api.cu:124)
thread_local std::string g_text;        // storage for returned strings

struct Ieee14Bus { const char* id; double kv; int type; double vset, p, q; };
struct Ieee14Branch { const char* id; const char* from; const char* to; double r, x, b, g, tap, shift; int xfmr; };
struct Ieee14Meas { const char* id; int type; const char* loc; int end; double sigma; int pseudo; };
#include "ieee14_data.inc"

inline Engine* E(SLE_Handle h) { return reinterpret_cast<Engine*>(h); }

SLE_StatusCode fail(SLE_StatusCode code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

void cfg_from_c(const SLE_Config* c, EngineConfig& e) {
    e.device_id = c->device_id;
    e.max_buses = c->max_buses;
    e.max_branches = c->max_branches;
    e.max_measurements = c->max_measurements;
    e.max_switching_devices = c->max_switching_devices;
    e.enable_robust = c->enable_robust;
    e.huber_gamma = c->huber_gamma;
    e.convergence_tolerance = c->convergence_tolerance;
    e.max_realtime_iterations = c->max_realtime_iterations;
    e.max_precision_iterations = c->max_precision_iterations;
    e.realtime_time_limit_ms = c->realtime_time_limit_ms;
    e.use_flat_start_default = c->use_flat_start_default;
    e.enable_profiling = c->enable_profiling;
    e.use_cuda_graphs = c->use_cuda_graphs;
    e.block_size_standard = c->block_size_standard;
    e.block_size_reduction = c->block_size_reduction;
    e.use_double_precision = c->use_double_precision;
    e.voltage_min_pu = c->voltage_min_pu;
    e.voltage_max_pu = c->voltage_max_pu;
    e.bad_data_threshold = c->bad_data_threshold;
    e.auto_bad_data_rejection = c->auto_bad_data_rejection;
}

void cfg_to_c(const EngineConfig& e, SLE_Config* c) {
    std::memset(c, 0, sizeof(*c));
    c->device_id = e.device_id;
    c->max_buses = e.max_buses;
    c->max_branches = e.max_branches;
    c->max_measurements = e.max_measurements;
    c->max_switching_devices = e.max_switching_devices;
    c->enable_robust = e.enable_robust;
    c->huber_gamma = e.huber_gamma;
    c->convergence_tolerance = e.convergence_tolerance;
    c->max_realtime_iterations = e.max_realtime_iterations;
    c->max_precision_iterations = e.max_precision_iterations;
    c->realtime_time_limit_ms = e.realtime_time_limit_ms;
    c->use_flat_start_default = e.use_flat_start_default;
    c->enable_profiling = e.enable_profiling;
    c->use_cuda_graphs = e.use_cuda_graphs;
    c->block_size_standard = e.block_size_standard;
    c->block_size_reduction = e.block_size_reduction;
    c->use_double_precision = e.use_double_precision;
    c->voltage_min_pu = e.voltage_min_pu;
    c->voltage_max_pu = e.voltage_max_pu;
    c->bad_data_threshold = e.bad_data_threshold;
    c->auto_bad_data_rejection = e.auto_bad_data_rejection;
}

// INI-style "key = value" file with optional [sections] and # / ; comments
// (reference include/sle_config.h:244-290).
bool parse_config(const std::string& text, EngineConfig& e) {
    std::istringstream in(text);
    std::string line;
    auto trim = [](std::string s) {
        const size_t a = s.find_first_not_of(" \t\r\n");
        if (a == std::string::npos) return std::string();
        const size_t b = s.find_last_not_of(" \t\r\n");
        return s.substr(a, b - a + 1);
    };
    auto as_bool = [](const std::string& v) { return v == "1" || v == "true" || v == "yes" || v == "on"; };
    while (std::getline(in, line)) {
        const size_t hash = line.find_first_of("#;");
        if (hash != std::string::npos) line = line.substr(0, hash);
        line = trim(line);
        if (line.empty() || line[0] == '[') continue;
        const size_t eq = line.find('=');
        if (eq == std::string::npos) continue;
        const std::string k = trim(line.substr(0, eq)), v = trim(line.substr(eq + 1));
        try {
            if (k == "device_id") e.device_id = std::stoi(v);
            else if (k == "max_buses") e.max_buses = std::stoull(v);
            else if (k == "max_branches") e.max_branches = std::stoull(v);
            else if (k == "max_measurements") e.max_measurements = std::stoull(v);
            else if (k == "max_switching_devices") e.max_switching_devices = std::stoull(v);
            else if (k == "enable_robust_estimation") e.enable_robust = as_bool(v);
            else if (k == "huber_gamma") e.huber_gamma = std::stod(v);
            else if (k == "convergence_tolerance") e.convergence_tolerance = std::stod(v);
            else if (k == "max_realtime_iterations") e.max_realtime_iterations = std::stoi(v);
            else if (k == "realtime_time_limit_ms") e.realtime_time_limit_ms = std::stod(v);
            else if (k == "max_precision_iterations") e.max_precision_iterations = std::stoi(v);
            else if (k == "use_flat_start_default") e.use_flat_start_default = as_bool(v);
            else if (k == "enable_profiling") e.enable_profiling = as_bool(v);
            else if (k == "use_cuda_graphs") e.use_cuda_graphs = as_bool(v);
            else if (k == "block_size_standard") e.block_size_standard = std::stoi(v);
            else if (k == "block_size_reduction") e.block_size_reduction = std::stoi(v);
            else if (k == "use_double_precision") e.use_double_precision = as_bool(v);
            else if (k == "voltage_min_pu") e.voltage_min_pu = std::stod(v);
            else if (k == "voltage_max_pu") e.voltage_max_pu = std::stod(v);
            else if (k == "bad_data_threshold") e.bad_data_threshold = std::stod(v);
            else if (k == "auto_bad_data_rejection") e.auto_bad_data_rejection = as_bool(v);
        } catch (...) {
            return false;
        }
    }
    return true;
}

std::string config_text(const EngineConfig& e) {
    std::ostringstream o;
    o.precision(17);
    o << "# SLE engine configuration\n[device]\ndevice_id = " << e.device_id << "\n\n[capacity]\nmax_buses = "
      << e.max_buses << "\nmax_branches = " << e.max_branches << "\nmax_measurements = " << e.max_measurements
      << "\nmax_switching_devices = " << e.max_switching_devices << "\n\n[solver]\nenable_robust_estimation = "
      << (e.enable_robust ? "true" : "false") << "\nhuber_gamma = " << e.huber_gamma
      << "\nconvergence_tolerance = " << e.convergence_tolerance
      << "\nmax_realtime_iterations = " << e.max_realtime_iterations
      << "\nrealtime_time_limit_ms = " << e.realtime_time_limit_ms
      << "\nmax_precision_iterations = " << e.max_precision_iterations
      << "\nuse_flat_start_default = " << (e.use_flat_start_default ? "true" : "false")
      << "\n\n[performance]\nenable_profiling = " << (e.enable_profiling ? "true" : "false")
      << "\nuse_cuda_graphs = " << (e.use_cuda_graphs ? "true" : "false")
      << "\nblock_size_standard = " << e.block_size_standard << "\nblock_size_reduction = " << e.block_size_reduction
      << "\n\n[numerical]\nuse_double_precision = " << (e.use_double_precision ? "true" : "false")
      << "\nvoltage_min_pu = " << e.voltage_min_pu << "\nvoltage_max_pu = " << e.voltage_max_pu
      << "\n\n[bad_data]\nbad_data_threshold = " << e.bad_data_threshold
      << "\nauto_bad_data_rejection = " << (e.auto_bad_data_rejection ? "true" : "false") << "\n";
    return o.str();
}

bool read_file(const char* path, std::string& out) {
    std::ifstream f(path);
    if (!f) return false;
    std::ostringstream s;
    s << f.rdbuf();
    out = s.str();
    return true;
}

SLE_StatusCode status_from_result(const sle_gb300::SolveResult& r) {
    switch (r.status) {  // sle_api.cu:971-984
        case sle_gb300::CONV_OK: return SLE_OK;
        case sle_gb300::CONV_MAXIT: return SLE_ERROR_MAX_ITERATIONS;
        case sle_gb300::CONV_DIVERGED: return SLE_ERROR_DIVERGED;
        case sle_gb300::CONV_SINGULAR: return SLE_ERROR_SINGULAR_MATRIX;
        case sle_gb300::CONV_NOTOBS: return SLE_ERROR_NOT_OBSERVABLE;
        default: return SLE_ERROR_UNKNOWN;
    }
}

void result_to_c(const sle_gb300::SolveResult& r, SLE_Result* c) {
    c->status = static_cast<SLE_ConvergenceStatus>(r.status);
    c->iterations = r.iterations;
    c->max_mismatch = r.max_mismatch;
    c->objective = r.objective;
    c->computation_time_ms = r.time_ms;
    c->largest_residual = r.largest_residual;
    c->largest_residual_idx = r.largest_idx;
    c->bad_data_count = r.bad_count;
}

inline bool is_bus_meas(int t) { return t == 0 || t == 1 || t == 2 || t == 3 || t == 7 || t == 8; }

SLE_StatusCode do_solve(Engine* e, const sle_gb300::SolveRequest& rq, SLE_Result* result,
                        sle_gb300::SolveResult& out) {
    const int32_t rc = e->solve(rq, out);
    if (rc != 0 || out.status == sle_gb300::CONV_NOTOBS) g_last_error = e->last_error;
    if (result) result_to_c(out, result);
    return SLE_OK;
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------- lifecycle
SLE_API SLE_StatusCode SLE_CALL sle_Create(SLE_Handle* handle) {
    if (!handle) return SLE_ERROR_INVALID_ARGUMENT;
    try {
        *handle = reinterpret_cast<SLE_Handle>(new Engine(EngineConfig()));
    } catch (...) {
        return fail(SLE_ERROR_OUT_OF_MEMORY, "Failed to create engine");
    }
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_CreateWithConfig(SLE_Handle* handle, const SLE_Config* config) {
    if (!handle || !config) return SLE_ERROR_INVALID_ARGUMENT;
    EngineConfig c;
    cfg_from_c(config, c);
    try {
        *handle = reinterpret_cast<SLE_Handle>(new Engine(c));
    } catch (...) {
        return fail(SLE_ERROR_OUT_OF_MEMORY, "Failed to create engine with config");
    }
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_CreateFromConfigFile(SLE_Handle* handle, const char* path) {
    if (!handle || !path) return SLE_ERROR_INVALID_ARGUMENT;
    std::string text;
    EngineConfig c;
    if (!read_file(path, text) || !parse_config(text, c)) return fail(SLE_ERROR_CONFIG_FILE, "Cannot read config file");
    auto* e = new Engine(c);
    e->config_path = path;
    *handle = reinterpret_cast<SLE_Handle>(e);
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_Initialize(SLE_Handle handle) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    const int32_t rc = E(handle)->initialize();
    if (rc) return fail(SLE_ERROR_CUDA_FAILURE, E(handle)->last_error);
    return SLE_OK;
}

SLE_API void SLE_CALL sle_Destroy(SLE_Handle handle) { delete E(handle); }

// ------------------------------------------------------------ configuration
SLE_API SLE_StatusCode SLE_CALL sle_LoadConfigFile(const char* path, SLE_Config* config) {
    if (!path || !config) return SLE_ERROR_INVALID_ARGUMENT;
    std::string text;
    EngineConfig c;
    if (!read_file(path, text) || !parse_config(text, c)) return fail(SLE_ERROR_CONFIG_FILE, "Cannot read config file");
    cfg_to_c(c, config);
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_SaveConfigFile(const char* path, const SLE_Config* config) {
    if (!path || !config) return SLE_ERROR_INVALID_ARGUMENT;
    EngineConfig c;
    cfg_from_c(config, c);
    std::ofstream f(path);
    if (!f) return fail(SLE_ERROR_CONFIG_FILE, "Cannot write config file");
    f << config_text(c);
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_ReloadConfigFromFile(SLE_Handle handle, const char* path) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    if (!path) return SLE_ERROR_INVALID_ARGUMENT;
    std::string text;
    EngineConfig c = E(handle)->cfg;
    if (!read_file(path, text) || !parse_config(text, c)) return fail(SLE_ERROR_CONFIG_FILE, "Cannot read config file");
    // solver settings only; capacity and device stay (sle_api.h: "Only affects solver settings")
    c.device_id = E(handle)->cfg.device_id;
    E(handle)->cfg = c;
    E(handle)->config_path = path;
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_ReloadConfig(SLE_Handle handle) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    const std::string p = E(handle)->config_path.empty() ? std::string("sle_engine.config") : E(handle)->config_path;
    return sle_ReloadConfigFromFile(handle, p.c_str());
}

SLE_API const char* SLE_CALL sle_GetDefaultConfigPath(void) { return "sle_engine.config"; }

SLE_API const char* SLE_CALL sle_GetConfigPath(SLE_Handle handle) {
    if (!handle) return "";
    g_text = E(handle)->config_path;
    return g_text.c_str();
}

SLE_API SLE_StatusCode SLE_CALL sle_EnsureConfigFile(const char* path) {
    const char* p = path ? path : "sle_engine.config";
    std::ifstream chk(p);
    if (chk) return SLE_OK;
    std::ofstream f(p);
    if (!f) return fail(SLE_ERROR_CONFIG_FILE, "Cannot create config file");
    f << config_text(EngineConfig());
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_GetConfig(SLE_Handle handle, SLE_Config* config) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    if (!config) return SLE_ERROR_INVALID_ARGUMENT;
    cfg_to_c(E(handle)->cfg, config);
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_SetConfig(SLE_Handle handle, const SLE_Config* config) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    if (!config) return SLE_ERROR_INVALID_ARGUMENT;
    EngineConfig c = E(handle)->cfg;
    cfg_from_c(config, c);
    c.device_id = E(handle)->cfg.device_id;  // device is fixed after creation
    if (c.use_double_precision != E(handle)->cfg.use_double_precision) E(handle)->model.structure_dirty = true;
    E(handle)->cfg = c;
    return SLE_OK;
}

// ------------------------------------------------------------------- errors
SLE_API const char* SLE_CALL sle_GetLastError(SLE_Handle handle) {
    (void)handle;
    return g_last_error.c_str();
}

SLE_API const char* SLE_CALL sle_GetDeviceInfo(SLE_Handle handle) {
    if (!handle) return "";
    g_text = E(handle)->device_info();
    return g_text.c_str();
}

// ------------------------------------------------------------ model building
SLE_API SLE_StatusCode SLE_CALL sle_AddBus(SLE_Handle handle, const SLE_BusInfo* info) {
    if (!handle || !info || !info->id) return SLE_ERROR_INVALID_ARGUMENT;
    const int32_t r = E(handle)->model.add_bus(info->id, info->base_kv, info->type, info->v_setpoint,
                                               info->p_scheduled, info->q_scheduled);
    if (r < 0) return fail(SLE_ERROR_DUPLICATE_ID, "Failed to add bus - duplicate ID or invalid");
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_AddBuses(SLE_Handle handle, const SLE_BusInfo* buses, int32_t count) {
    if (!handle || !buses || count <= 0) return SLE_ERROR_INVALID_ARGUMENT;
    for (int32_t i = 0; i < count; ++i) {
        const SLE_StatusCode s = sle_AddBus(handle, &buses[i]);
        if (s != SLE_OK) return s;
    }
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_AddBranch(SLE_Handle handle, const SLE_BranchInfo* info) {
    if (!handle || !info || !info->id || !info->from_bus || !info->to_bus) return SLE_ERROR_INVALID_ARGUMENT;
    const int32_t r = E(handle)->model.add_branch(info->id, info->from_bus, info->to_bus, info->resistance,
                                                  info->reactance, info->susceptance, info->conductance,
                                                  info->tap_ratio, info->phase_shift, info->is_transformer,
                                                  info->sd_id ? info->sd_id : "");
    if (r < 0) return fail(SLE_ERROR_ELEMENT_NOT_FOUND, "Failed to add branch - bus not found or duplicate ID");
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_AddBranches(SLE_Handle handle, const SLE_BranchInfo* br, int32_t count) {
    if (!handle || !br || count <= 0) return SLE_ERROR_INVALID_ARGUMENT;
    for (int32_t i = 0; i < count; ++i) {
        const SLE_StatusCode s = sle_AddBranch(handle, &br[i]);
        if (s != SLE_OK) return s;
    }
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_AddMeasurement(SLE_Handle handle, const SLE_MeasurementInfo* info) {
    if (!handle || !info || !info->id || !info->location) return SLE_ERROR_INVALID_ARGUMENT;
    const int32_t r = E(handle)->model.add_measurement(info->id, info->type, info->location, info->branch_end,
                                                       info->sigma, info->pt_ratio, info->ct_ratio, info->is_pseudo);
    if (r < 0) return fail(SLE_ERROR_ELEMENT_NOT_FOUND, "Failed to add measurement - location not found");
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_AddMeasurements(SLE_Handle handle, const SLE_MeasurementInfo* m, int32_t count) {
    if (!handle || !m || count <= 0) return SLE_ERROR_INVALID_ARGUMENT;
    for (int32_t i = 0; i < count; ++i) {
        const SLE_StatusCode s = sle_AddMeasurement(handle, &m[i]);
        if (s != SLE_OK) return s;
    }
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_AddSwitch(SLE_Handle handle, const SLE_SwitchInfo* info) {
    if (!handle || !info || !info->id || !info->branch_id) return SLE_ERROR_INVALID_ARGUMENT;
    const int32_t r = E(handle)->model.add_switch(info->id, info->branch_id, info->status == SLE_SWITCH_CLOSED);
    if (r < 0) return fail(SLE_ERROR_ELEMENT_NOT_FOUND, "Failed to add switch - branch not found or duplicate ID");
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_RemoveBus(SLE_Handle handle, const char* bus_id) {
    if (!handle || !bus_id) return SLE_ERROR_INVALID_ARGUMENT;
    if (E(handle)->uploaded()) E(handle)->download_results();
    if (E(handle)->model.remove_bus(bus_id) < 0) return fail(SLE_ERROR_ELEMENT_NOT_FOUND, "Bus not found");
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_RemoveBranch(SLE_Handle handle, const char* branch_id) {
    if (!handle || !branch_id) return SLE_ERROR_INVALID_ARGUMENT;
    if (E(handle)->uploaded()) E(handle)->download_results();
    if (E(handle)->model.remove_branch(branch_id) < 0) return fail(SLE_ERROR_ELEMENT_NOT_FOUND, "Branch not found");
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_UpdateBranch(SLE_Handle handle, const SLE_BranchInfo* info) {
    if (!handle || !info || !info->id) return SLE_ERROR_INVALID_ARGUMENT;
    auto& M = E(handle)->model;
    const int32_t k = M.find_branch(info->id);
    if (k < 0) return fail(SLE_ERROR_ELEMENT_NOT_FOUND, "Branch not found");
    bool moved = false;
    if (info->from_bus && info->to_bus) {
        const int32_t f = M.find_bus(info->from_bus), t = M.find_bus(info->to_bus);
        if (f < 0 || t < 0) return fail(SLE_ERROR_ELEMENT_NOT_FOUND, "Bus not found");
        moved = f != M.br_from[k] || t != M.br_to[k];
        M.br_from[k] = f;
        M.br_to[k] = t;
    }
    M.br_r[k] = info->resistance;
    M.br_x[k] = info->reactance;
    M.br_b[k] = info->susceptance;
    M.br_g[k] = info->conductance;
    M.br_tap[k] = info->tap_ratio;
    M.br_shift[k] = info->phase_shift;
    M.br_xfmr[k] = info->is_transformer;
    if (moved)
        M.structure_dirty = true;  // new endpoints: a new pattern
    else
        M.branch_values_dirty = true;
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_SetTransformerTap(SLE_Handle handle, const char* id, SLE_Real tap) {
    if (!handle || !id) return SLE_ERROR_INVALID_ARGUMENT;
    if (tap <= 0) return fail(SLE_ERROR_INVALID_ARGUMENT, "Tap ratio must be positive");
    auto& M = E(handle)->model;
    const int32_t k = M.find_branch(id);
    if (k < 0) return fail(SLE_ERROR_ELEMENT_NOT_FOUND, "Branch not found");
    M.br_tap[k] = tap;
    M.branch_values_dirty = true;  // parameter edit: values only, applied on the device
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_SetTransformerPhaseShift(SLE_Handle handle, const char* id, SLE_Real shift) {
    if (!handle || !id) return SLE_ERROR_INVALID_ARGUMENT;
    auto& M = E(handle)->model;
    const int32_t k = M.find_branch(id);
    if (k < 0) return fail(SLE_ERROR_ELEMENT_NOT_FOUND, "Branch not found");
    M.br_shift[k] = shift;
    M.branch_values_dirty = true;  // parameter edit: values only, applied on the device
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_SetBranchImpedance(SLE_Handle handle, const char* id, SLE_Real r, SLE_Real x,
                                                       SLE_Real b, SLE_Real g) {
    if (!handle || !id) return SLE_ERROR_INVALID_ARGUMENT;
    auto& M = E(handle)->model;
    const int32_t k = M.find_branch(id);
    if (k < 0) return fail(SLE_ERROR_ELEMENT_NOT_FOUND, "Branch not found");
    M.br_r[k] = r;
    M.br_x[k] = x;
    M.br_b[k] = b;
    M.br_g[k] = g;
    M.branch_values_dirty = true;  // parameter edit: values only, applied on the device
    return SLE_OK;
}

SLE_API SLE_Real SLE_CALL sle_GetTransformerTap(SLE_Handle handle, const char* id) {
    if (!handle || !id) return 1.0;
    const int32_t k = E(handle)->model.find_branch(id);
    return k < 0 ? 1.0 : E(handle)->model.br_tap[k];
}

SLE_API SLE_Real SLE_CALL sle_GetTransformerPhaseShift(SLE_Handle handle, const char* id) {
    if (!handle || !id) return 0.0;
    const int32_t k = E(handle)->model.find_branch(id);
    return k < 0 ? 0.0 : E(handle)->model.br_shift[k];
}

// ------------------------------------------------------------------- meters
SLE_API SLE_StatusCode SLE_CALL sle_AddMeter(SLE_Handle handle, const SLE_MeterInfo* info) {
    if (!handle || !info || !info->id || !info->bus_id) return SLE_ERROR_INVALID_ARGUMENT;
    sle_gb300::Meter m;
    m.id = info->id;
    m.type = info->type;
    m.end = info->branch_end;
    m.pt = info->pt_ratio;
    m.ct = info->ct_ratio;
    m.sigma_v = info->sigma_v;
    m.sigma_p = info->sigma_p;
    m.sigma_i = info->sigma_i;
    const int32_t r = E(handle)->model.add_meter(m, info->bus_id, info->branch_id ? info->branch_id : "");
    if (r < 0) return fail(SLE_ERROR_ELEMENT_NOT_FOUND, "Failed to add meter");
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_UpdateMeterReading(SLE_Handle handle, const char* meter_id, const char* channel,
                                                       SLE_Real value) {
    if (!handle || !meter_id || !channel) return SLE_ERROR_INVALID_ARGUMENT;
    auto& M = E(handle)->model;
    const int32_t mi = M.find_meter(meter_id);
    if (mi < 0) return fail(SLE_ERROR_ELEMENT_NOT_FOUND, "Meter not found");
    const int32_t q = sle_gb300::Model::channel_meas(M.meters[mi], channel);
    if (q < 0) return fail(SLE_ERROR_INVALID_ARGUMENT, "Meter has no such channel");
    M.m_value[q] = value;
    M.values_dirty = true;
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_UpdateMeterReadings(SLE_Handle handle, const SLE_MeterReading* rd, int32_t count,
                                                        int32_t sync) {
    if (!handle || !rd || count <= 0) return SLE_ERROR_INVALID_ARGUMENT;
    for (int32_t i = 0; i < count; ++i) {
        const SLE_StatusCode s = sle_UpdateMeterReading(handle, rd[i].meter_id, rd[i].channel, rd[i].value);
        if (s != SLE_OK) return s;
    }
    if (sync) return sle_SyncMeasurementsToDevice(handle);
    return SLE_OK;
}

static SLE_StatusCode meter_value(SLE_Handle handle, const char* meter_id, const char* channel, SLE_Real* out,
                                  int which) {
    if (!handle || !meter_id || !channel || !out) return SLE_ERROR_INVALID_ARGUMENT;
    Engine* e = E(handle);
    auto& M = e->model;
    const int32_t mi = M.find_meter(meter_id);
    if (mi < 0) return fail(SLE_ERROR_ELEMENT_NOT_FOUND, "Meter not found");
    const int32_t q = sle_gb300::Model::channel_meas(M.meters[mi], channel);
    if (q < 0) return fail(SLE_ERROR_INVALID_ARGUMENT, "Meter has no such channel");
    if (which) e->download_results(Engine::DL_MEAS);
    *out = which == 0 ? M.m_value[q] : (which == 1 ? M.m_est[q] : M.m_res[q]);
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_GetMeterReading(SLE_Handle h, const char* id, const char* ch, SLE_Real* v) {
    return meter_value(h, id, ch, v, 0);
}
SLE_API SLE_StatusCode SLE_CALL sle_GetMeterEstimate(SLE_Handle h, const char* id, const char* ch, SLE_Real* v) {
    return meter_value(h, id, ch, v, 1);
}
SLE_API SLE_StatusCode SLE_CALL sle_GetMeterResidual(SLE_Handle h, const char* id, const char* ch, SLE_Real* v) {
    return meter_value(h, id, ch, v, 2);
}

// -------------------------------------------------------------- device data
SLE_API SLE_StatusCode SLE_CALL sle_UploadModel(SLE_Handle handle) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    if (E(handle)->upload() != 0) return fail(SLE_ERROR_CUDA_FAILURE, "Failed to upload model to GPU: " + E(handle)->last_error);
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_UpdateTelemetry(SLE_Handle handle, const SLE_Real* values, int32_t count) {
    if (!handle || !values || count <= 0) return SLE_ERROR_INVALID_ARGUMENT;
    Engine* e = E(handle);
    if (!e->uploaded() || e->model.structure_dirty) {
        if (e->upload() != 0) return fail(SLE_ERROR_INVALID_ARGUMENT, "Failed to update telemetry: " + e->last_error);
    }
    if (e->update_telemetry(values, count) != 0) return fail(SLE_ERROR_INVALID_ARGUMENT, "Failed to update telemetry");
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_UpdateMeasurement(SLE_Handle handle, const char* id, SLE_Real value) {
    if (!handle || !id) return SLE_ERROR_INVALID_ARGUMENT;
    auto& M = E(handle)->model;
    const int32_t q = M.find_meas(id);
    if (q < 0) return fail(SLE_ERROR_ELEMENT_NOT_FOUND, "Measurement not found");
    M.m_value[q] = value;
    M.values_dirty = true;
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_UpdateMeasurementBatch(SLE_Handle handle, const SLE_MeasurementUpdate* up,
                                                           int32_t count, int32_t sync) {
    if (!handle || !up || count <= 0) return SLE_ERROR_INVALID_ARGUMENT;
    for (int32_t i = 0; i < count; ++i) {
        const SLE_StatusCode s = sle_UpdateMeasurement(handle, up[i].meas_id, up[i].value);
        if (s != SLE_OK) return s;
    }
    if (sync) return sle_SyncMeasurementsToDevice(handle);
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_SyncMeasurementsToDevice(SLE_Handle handle) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    if (E(handle)->sync_measurements() != 0) return fail(SLE_ERROR_CUDA_FAILURE, E(handle)->last_error);
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_GetMeasurementDetails(SLE_Handle handle, const char* id, SLE_MeasurementDetails* d) {
    if (!handle || !id || !d) return SLE_ERROR_INVALID_ARGUMENT;
    Engine* e = E(handle);
    auto& M = e->model;
    const int32_t q = M.find_meas(id);
    if (q < 0) return fail(SLE_ERROR_ELEMENT_NOT_FOUND, "Measurement not found");
    e->download_results(Engine::DL_MEAS);
    d->id = M.m_id[q].c_str();
    d->type = static_cast<SLE_MeasurementType>(M.m_type[q]);
    d->location_id = is_bus_meas(M.m_type[q]) ? M.bus_id[M.m_loc[q]].c_str() : M.br_id[M.m_loc[q]].c_str();
    d->branch_end = static_cast<SLE_BranchEnd>(M.m_end[q]);
    d->sigma = M.m_sigma[q];
    d->pt_ratio = M.m_pt[q];
    d->ct_ratio = M.m_ct[q];
    d->is_pseudo = M.m_pseudo[q];
    d->internal_index = q;
    d->current_value = M.m_value[q];
    d->estimated_value = M.m_est[q];
    d->residual = M.m_res[q];
    d->is_active = M.m_active[q];
    return SLE_OK;
}

SLE_API const char* SLE_CALL sle_GetMeasurementIdByIndex(SLE_Handle handle, int32_t index) {
    if (!handle) return nullptr;
    auto& M = E(handle)->model;
    M.ensure_names();
    if (index < 0 || index >= M.n_meas()) return nullptr;
    return M.m_id[index].c_str();
}

// ----------------------------------------------------------------- switches
SLE_API SLE_StatusCode SLE_CALL sle_SetSwitchStatus(SLE_Handle handle, const char* sd_id, SLE_SwitchStatus status) {
    if (!handle || !sd_id) return SLE_ERROR_INVALID_ARGUMENT;
    auto& M = E(handle)->model;
    const int32_t s = M.find_switch(sd_id);
    if (s < 0) return fail(SLE_ERROR_ELEMENT_NOT_FOUND, "Switch not found");
    // Queued in the reference (sle_engine.cu:568-580) and applied before the
    // next solve; here the status is recorded now and takes effect at the next
    // upload, which the next solve performs.
    // A switched branch is in the uploaded pattern, so the change is a value
    // edit applied on the device at the next solve (or by
    // sle_ApplySwitchChanges); a switch added after the analysis of an open
    // branch needs a new analysis.
    const uint8_t closed = status == SLE_SWITCH_CLOSED ? 1 : 0;
    if (M.sd_closed[s] != closed) {
        M.sd_closed[s] = closed;
        M.br_closed[M.sd_branch[s]] = closed;
        if (E(handle)->branch_in_pattern(M.sd_branch[s]))
            M.branch_values_dirty = true;
        else
            M.structure_dirty = true;
    }
    return SLE_OK;
}

SLE_API SLE_SwitchStatus SLE_CALL sle_GetSwitchStatus(SLE_Handle handle, const char* sd_id) {
    if (!handle || !sd_id) return SLE_SWITCH_OPEN;
    auto& M = E(handle)->model;
    const int32_t s = M.find_switch(sd_id);
    if (s < 0) return SLE_SWITCH_OPEN;
    return M.sd_closed[s] ? SLE_SWITCH_CLOSED : SLE_SWITCH_OPEN;
}

SLE_API SLE_StatusCode SLE_CALL sle_ApplySwitchChanges(SLE_Handle handle) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    Engine* e = E(handle);
    if (e->uploaded() && e->model.branch_values_dirty && !e->model.structure_dirty) {
        if (e->apply_branch_edits() != 0) return fail(SLE_ERROR_CUDA_FAILURE, e->last_error);
    }
    if (e->uploaded() && e->model.structure_dirty) {
        if (e->upload() != 0) return fail(SLE_ERROR_CUDA_FAILURE, e->last_error);
    }
    return SLE_OK;
}

// --------------------------------------------------------------- estimation
SLE_API SLE_StatusCode SLE_CALL sle_Solve(SLE_Handle handle, SLE_EstimationMode mode, SLE_Result* result) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    Engine* e = E(handle);
    sle_gb300::SolveRequest rq;  // sle_engine.cu:609-628
    rq.mode = mode == SLE_MODE_PRECISION ? sle_gb300::Mode::PRECISION : sle_gb300::Mode::REALTIME;
    if (rq.mode == sle_gb300::Mode::REALTIME) {
        rq.max_iterations = e->cfg.max_realtime_iterations;
        rq.time_limit_ms = e->cfg.realtime_time_limit_ms;
    } else {
        rq.max_iterations = e->cfg.max_precision_iterations;
        rq.time_limit_ms = 0.0;
    }
    rq.tolerance = e->cfg.convergence_tolerance;
    rq.robust = e->cfg.enable_robust;
    rq.huber_gamma = e->cfg.huber_gamma;
    rq.flat_start = e->cfg.use_flat_start_default;
    sle_gb300::SolveResult out;
    do_solve(e, rq, result, out);
    return status_from_result(out);
}

SLE_API SLE_StatusCode SLE_CALL sle_SolveWithConfig(SLE_Handle handle, const SLE_SolverConfig* c, SLE_Result* result) {
    if (!handle || !c) return SLE_ERROR_INVALID_ARGUMENT;
    Engine* e = E(handle);
    sle_gb300::SolveRequest rq;
    rq.mode = c->mode == SLE_MODE_PRECISION ? sle_gb300::Mode::PRECISION : sle_gb300::Mode::REALTIME;
    rq.max_iterations = c->max_iterations;
    rq.tolerance = c->tolerance;
    rq.huber_gamma = c->huber_gamma;
    rq.robust = c->use_robust;
    rq.flat_start = c->use_flat_start;
    rq.time_limit_ms = c->time_limit_ms;
    sle_gb300::SolveResult out;
    do_solve(e, rq, result, out);
    // sle_api.cu:1011 reports only converged / not converged
    return out.status == sle_gb300::CONV_OK ? SLE_OK : SLE_ERROR_MAX_ITERATIONS;
}

SLE_API SLE_StatusCode SLE_CALL sle_CheckObservability(SLE_Handle handle, int32_t* is_observable, int32_t* islands) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    // Topological check (sle_engine.cu:684-753): one island over the closed
    // branches and at least as many active rows as states.  On an uploaded
    // model the islands are labelled on the device; before the first upload
    // the host model is checked the same way.
    Engine* en = E(handle);
    auto& M = en->model;
    const int32_t n = M.n_bus();
    int32_t count = 0, active = 0;
    if (en->uploaded() && !M.structure_dirty && M.branch_values_dirty && !en->batch_mode()) {
        if (en->apply_branch_edits() != 0) return fail(SLE_ERROR_CUDA_FAILURE, en->last_error);
    }
    if (en->uploaded() && !M.structure_dirty && !en->batch_mode()) {
        if (en->check_islands(&count, &active) != 0) return fail(SLE_ERROR_CUDA_FAILURE, en->last_error);
    } else {
        std::vector<int32_t> par(n);
        for (int32_t i = 0; i < n; ++i) par[i] = i;
        auto find = [&](int32_t x) {
            while (par[x] != x) x = par[x] = par[par[x]];
            return x;
        };
        for (int32_t k = 0; k < M.n_branch(); ++k)
            if (M.br_closed[k]) {
                const int32_t a = find(M.br_from[k]), b = find(M.br_to[k]);
                if (a != b) par[a] = b;
            }
        for (int32_t i = 0; i < n; ++i) count += (find(i) == i);
        for (int32_t q = 0; q < M.n_meas(); ++q) active += M.m_active[q];
    }
    const bool obs = n > 0 && count == 1 && active >= 2 * n - 1;
    if (is_observable) *is_observable = obs ? 1 : 0;
    if (islands) *islands = count;
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_ApplyFlatStart(SLE_Handle handle) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    if (E(handle)->flat_start() != 0) return fail(SLE_ERROR_CUDA_FAILURE, E(handle)->last_error);
    return SLE_OK;
}

// ------------------------------------------------------------------ results
static SLE_StatusCode copy_bus(SLE_Handle handle, SLE_Real* out, int32_t count, bool angle) {
    if (!handle || !out || count <= 0) return SLE_ERROR_INVALID_ARGUMENT;
    Engine* e = E(handle);
    if (e->download_results(Engine::DL_STATE) != 0) return fail(SLE_ERROR_CUDA_FAILURE, e->last_error);
    const auto& src = angle ? e->model.bus_th : e->model.bus_v;
    const int32_t n = std::min<int32_t>(count, static_cast<int32_t>(src.size()));
    if (n > 0) std::memcpy(out, src.data(), sizeof(double) * n);
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_GetVoltageMagnitudes(SLE_Handle h, SLE_Real* v, int32_t c) { return copy_bus(h, v, c, false); }
SLE_API SLE_StatusCode SLE_CALL sle_GetVoltageAngles(SLE_Handle h, SLE_Real* v, int32_t c) { return copy_bus(h, v, c, true); }

SLE_API SLE_Real SLE_CALL sle_GetBusVoltage(SLE_Handle handle, const char* bus_id) {
    if (!handle || !bus_id) return 0.0;
    Engine* e = E(handle);
    const int32_t i = e->model.find_bus(bus_id);
    if (i < 0) return 0.0;
    e->download_results(Engine::DL_STATE);
    return e->model.bus_v[i];
}

SLE_API SLE_Real SLE_CALL sle_GetBusAngle(SLE_Handle handle, const char* bus_id) {
    if (!handle || !bus_id) return 0.0;
    Engine* e = E(handle);
    const int32_t i = e->model.find_bus(bus_id);
    if (i < 0) return 0.0;
    e->download_results(Engine::DL_STATE);
    return e->model.bus_th[i];
}

SLE_API SLE_StatusCode SLE_CALL sle_GetPowerInjections(SLE_Handle handle, SLE_Real* p, SLE_Real* q, int32_t count) {
    if (!handle || count <= 0) return SLE_ERROR_INVALID_ARGUMENT;
    Engine* e = E(handle);
    if (e->download_results(Engine::DL_FLOWS) != 0) return fail(SLE_ERROR_CUDA_FAILURE, e->last_error);
    const int32_t n = std::min<int32_t>(count, static_cast<int32_t>(e->p_inj.size()));
    if (p && n > 0) std::memcpy(p, e->p_inj.data(), sizeof(double) * n);
    if (q && n > 0) std::memcpy(q, e->q_inj.data(), sizeof(double) * n);
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_GetBranchFlows(SLE_Handle handle, SLE_Real* pf, SLE_Real* qf, SLE_Real* pt,
                                                   SLE_Real* qt, int32_t count) {
    if (!handle || count <= 0) return SLE_ERROR_INVALID_ARGUMENT;
    Engine* e = E(handle);
    if (e->download_results(Engine::DL_FLOWS) != 0) return fail(SLE_ERROR_CUDA_FAILURE, e->last_error);
    const int32_t n = std::min<int32_t>(count, static_cast<int32_t>(e->pf.size()));
    if (n > 0) {
        if (pf) std::memcpy(pf, e->pf.data(), sizeof(double) * n);
        if (qf) std::memcpy(qf, e->qf.data(), sizeof(double) * n);
        if (pt) std::memcpy(pt, e->pt.data(), sizeof(double) * n);
        if (qt) std::memcpy(qt, e->qt.data(), sizeof(double) * n);
    }
    return SLE_OK;
}

static SLE_Real branch_pq(SLE_Handle handle, const char* id, SLE_BranchEnd end, bool q) {
    if (!handle || !id) return std::nan("");
    Engine* e = E(handle);
    const int32_t k = e->model.find_branch(id);
    if (k < 0 || k >= static_cast<int32_t>(e->pf.size())) return std::nan("");
    e->download_results(Engine::DL_FLOWS);
    if (end == SLE_BRANCH_FROM) return q ? e->qf[k] : e->pf[k];
    return q ? e->qt[k] : e->pt[k];
}

SLE_API SLE_Real SLE_CALL sle_GetBranchP(SLE_Handle h, const char* id, SLE_BranchEnd end) { return branch_pq(h, id, end, false); }
SLE_API SLE_Real SLE_CALL sle_GetBranchQ(SLE_Handle h, const char* id, SLE_BranchEnd end) { return branch_pq(h, id, end, true); }

SLE_API SLE_StatusCode SLE_CALL sle_GetBusResiduals(SLE_Handle handle, const char* bus_id, SLE_Real* vr, SLE_Real* pr,
                                                    SLE_Real* qr, int32_t* count) {
    if (!handle || !bus_id) return SLE_ERROR_INVALID_ARGUMENT;
    Engine* e = E(handle);
    auto& M = e->model;
    const int32_t b = M.find_bus(bus_id);
    if (b < 0) return fail(SLE_ERROR_ELEMENT_NOT_FOUND, "Bus not found");
    e->download_results(Engine::DL_MEAS);
    int32_t c = 0;
    if (vr) *vr = 0.0;
    if (pr) *pr = 0.0;
    if (qr) *qr = 0.0;
    for (int32_t q = 0; q < M.n_meas(); ++q) {
        if (!is_bus_meas(M.m_type[q]) || M.m_loc[q] != b) continue;
        const int32_t t = M.m_type[q];
        if (t == 0 && vr) *vr = M.m_res[q];
        if ((t == 2 || t == 7) && pr) *pr = M.m_res[q];
        if ((t == 3 || t == 8) && qr) *qr = M.m_res[q];
        ++c;
    }
    if (count) *count = c;
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_GetBranchResiduals(SLE_Handle handle, const char* branch_id, SLE_BranchEnd end,
                                                       SLE_Real* pr, SLE_Real* qr, SLE_Real* ir, int32_t* count) {
    if (!handle || !branch_id) return SLE_ERROR_INVALID_ARGUMENT;
    Engine* e = E(handle);
    auto& M = e->model;
    const int32_t k = M.find_branch(branch_id);
    if (k < 0) return fail(SLE_ERROR_ELEMENT_NOT_FOUND, "Branch not found");
    e->download_results(Engine::DL_MEAS);
    int32_t c = 0;
    if (pr) *pr = 0.0;
    if (qr) *qr = 0.0;
    if (ir) *ir = 0.0;
    for (int32_t q = 0; q < M.n_meas(); ++q) {
        if (is_bus_meas(M.m_type[q]) || M.m_loc[q] != k || M.m_end[q] != end) continue;
        const int32_t t = M.m_type[q];
        if (t == 4 && pr) *pr = M.m_res[q];
        if (t == 5 && qr) *qr = M.m_res[q];
        if (t == 6 && ir) *ir = M.m_res[q];
        ++c;
    }
    if (count) *count = c;
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_GetResiduals(SLE_Handle handle, SLE_Real* values, int32_t count) {
    if (!handle || !values || count <= 0) return SLE_ERROR_INVALID_ARGUMENT;
    Engine* e = E(handle);
    if (e->download_results(Engine::DL_MEAS) != 0) return fail(SLE_ERROR_CUDA_FAILURE, e->last_error);
    const int32_t n = std::min<int32_t>(count, e->model.n_meas());
    if (n > 0) std::memcpy(values, e->model.m_res.data(), sizeof(double) * n);
    return SLE_OK;
}

SLE_API SLE_Real SLE_CALL sle_GetObjective(SLE_Handle handle) {
    if (!handle) return 0.0;
    return E(handle)->last_result().objective;
}

SLE_API SLE_StatusCode SLE_CALL sle_IdentifyBadData(SLE_Handle handle, SLE_Real threshold, int32_t* indices,
                                                    int32_t max_count, int32_t* actual_count) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    Engine* e = E(handle);
    e->download_results(Engine::DL_MEAS);
    const double thr = threshold > 0 ? threshold : e->cfg.bad_data_threshold;  // sle_engine.cu:959-977
    const auto& M = e->model;
    int32_t found = 0;
    for (int32_t q = 0; q < M.n_meas(); ++q) {
        if (M.m_active[q] && M.m_sigma[q] > 0 && std::fabs(M.m_res[q]) / M.m_sigma[q] > thr) {
            if (indices && found < max_count) indices[found] = q;
            ++found;
        }
    }
    if (actual_count) *actual_count = found;
    return SLE_OK;
}

// -------------------------------------------------------------- model info
SLE_API int32_t SLE_CALL sle_GetBusCount(SLE_Handle h) { return h ? E(h)->model.n_bus() : 0; }
SLE_API int32_t SLE_CALL sle_GetBranchCount(SLE_Handle h) { return h ? E(h)->model.n_branch() : 0; }
SLE_API int32_t SLE_CALL sle_GetMeasurementCount(SLE_Handle h) { return h ? E(h)->model.n_meas() : 0; }
SLE_API int32_t SLE_CALL sle_GetMeterCount(SLE_Handle h) { return h ? static_cast<int32_t>(E(h)->model.meters.size()) : 0; }
SLE_API size_t SLE_CALL sle_GetGPUMemoryUsage(SLE_Handle h) { return h ? E(h)->device_bytes() : 0; }
SLE_API SLE_Real SLE_CALL sle_GetLastSolveTime(SLE_Handle h) { return h ? E(h)->last_solve_ms() : 0.0; }

// ------------------------------------------------------------ test case etc.
SLE_API SLE_StatusCode SLE_CALL sle_LoadIEEE14Bus(SLE_Handle handle) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    for (const auto& b : kIeee14Buses) {
        SLE_BusInfo bi{b.id, b.kv, static_cast<SLE_BusType>(b.type), b.vset, b.p, b.q};
        sle_AddBus(handle, &bi);
    }
    for (const auto& b : kIeee14Branches) {
        SLE_BranchInfo bi{b.id, b.from, b.to, b.r, b.x, b.b, b.g, b.tap, b.shift, b.xfmr, nullptr};
        sle_AddBranch(handle, &bi);
    }
    for (const auto& m : kIeee14Meas) {
        SLE_MeasurementInfo mi{m.id, static_cast<SLE_MeasurementType>(m.type), m.loc,
                               static_cast<SLE_BranchEnd>(m.end), m.sigma, 1.0, 1.0, m.pseudo};
        sle_AddMeasurement(handle, &mi);
    }
    return SLE_OK;
}

SLE_API const char* SLE_CALL sle_GetVersion(void) { return SLE_VERSION_STRING; }

SLE_API int32_t SLE_CALL sle_GetCUDAVersion(void) {
    int v = 0;
    cudaRuntimeGetVersion(&v);
    return v;
}

SLE_API int32_t SLE_CALL sle_IsGPUAvailable(void) {
    int n = 0;
    return (cudaGetDeviceCount(&n) == cudaSuccess && n > 0) ? 1 : 0;
}

// ======================================================= sle_Ex extensions
SLE_API int32_t SLE_CALL sle_ExRealSize(void) { return static_cast<int32_t>(sizeof(SLE_Real)); }

SLE_API SLE_StatusCode SLE_CALL sle_ExLoadNetwork(SLE_Handle handle, int32_t n_bus, const int32_t* bus_type,
                                                  const SLE_Real* v_setpoint, int32_t n_branch, const int32_t* from,
                                                  const int32_t* to, const SLE_Real* r, const SLE_Real* x,
                                                  const SLE_Real* b, const SLE_Real* tap, const SLE_Real* shift,
                                                  const int32_t* status, int32_t n_meas, const int32_t* mtype,
                                                  const int32_t* mloc, const int32_t* mend, const SLE_Real* sigma,
                                                  const SLE_Real* z) {
    if (!handle || n_bus <= 0 || !bus_type || !v_setpoint || n_branch < 0 || n_meas < 0) return SLE_ERROR_INVALID_ARGUMENT;
    if (n_branch > 0 && (!from || !to || !r || !x || !b || !tap || !shift)) return SLE_ERROR_INVALID_ARGUMENT;
    if (n_meas > 0 && (!mtype || !mloc || !mend || !sigma || !z)) return SLE_ERROR_INVALID_ARGUMENT;
    for (int32_t i = 0; i < n_bus; ++i)
        if (bus_type[i] < 0 || bus_type[i] > 2) return fail(SLE_ERROR_INVALID_ARGUMENT, "invalid bus type");
    for (int32_t k = 0; k < n_branch; ++k)
        if (from[k] < 0 || from[k] >= n_bus || to[k] < 0 || to[k] >= n_bus)
            return fail(SLE_ERROR_ELEMENT_NOT_FOUND, "branch references an unknown bus");
    for (int32_t q = 0; q < n_meas; ++q) {
        if (mtype[q] < 0 || mtype[q] > 8) return fail(SLE_ERROR_INVALID_ARGUMENT, "invalid measurement type");
        const int32_t lim = is_bus_meas(mtype[q]) ? n_bus : n_branch;
        if (mloc[q] < 0 || mloc[q] >= lim) return fail(SLE_ERROR_ELEMENT_NOT_FOUND, "measurement location out of range");
    }
    E(handle)->model.load_soa(n_bus, bus_type, v_setpoint, n_branch, from, to, r, x, b, tap, shift, status, n_meas,
                              mtype, mloc, mend, sigma, z);
    return SLE_OK;
}

// ---- serving runtime ----------------------------------------------------------
struct SLE_ExServer {
    sle_gb300::Server srv;
    std::string err;
    explicit SLE_ExServer(const sle_gb300::ServeConfig& c) : srv(c) {}
};

static SLE_StatusCode server_rc(SLE_ExServer* s, int32_t rc) {
    if (rc == 0) return SLE_OK;
    s->err = s->srv.last_error;
    if (rc == -4) return fail(SLE_ERROR_INVALID_ARGUMENT, s->err);
    if (rc == -11) return fail(SLE_ERROR_ELEMENT_NOT_FOUND, s->err);
    if (rc == -5) return fail(SLE_ERROR_MODEL_INCOMPLETE, s->err);
    if (rc == -10) return fail(SLE_ERROR_OUT_OF_MEMORY, s->err);
    return fail(SLE_ERROR_CUDA_FAILURE, s->err);
}

SLE_API void SLE_CALL sle_ExServerDefaultConfig(SLE_ExServerConfig* c) {
    if (!c) return;
    const sle_gb300::ServeConfig d;
    c->use_double_precision = d.use_double_precision;
    c->max_iterations = d.max_iterations;
    c->tolerance = d.tolerance;
    c->robust = d.robust;
    c->huber_gamma = d.huber_gamma;
    for (int i = 0; i < 4; ++i) c->bucket_bus[i] = d.bucket_bus[i];
    c->own_unit_bus = d.own_unit_bus;
    c->device_id = d.device_id;
    c->memory_budget = d.memory_budget;
}

SLE_API SLE_StatusCode SLE_CALL sle_ExServerCreate(SLE_ExServer** out, const SLE_ExServerConfig* c) {
    if (!out) return SLE_ERROR_INVALID_ARGUMENT;
    sle_gb300::ServeConfig sc;
    if (c) {
        sc.use_double_precision = c->use_double_precision;
        sc.max_iterations = c->max_iterations > 0 ? c->max_iterations : sc.max_iterations;
        sc.tolerance = c->tolerance > 0.0 ? c->tolerance : sc.tolerance;
        sc.robust = c->robust;
        sc.huber_gamma = c->huber_gamma > 0.0 ? c->huber_gamma : sc.huber_gamma;
        for (int i = 0; i < 4; ++i) sc.bucket_bus[i] = c->bucket_bus[i];
        sc.own_unit_bus = c->own_unit_bus > 0 ? c->own_unit_bus : sc.own_unit_bus;
        sc.device_id = c->device_id;
        sc.memory_budget = c->memory_budget;
    }
    *out = new SLE_ExServer(sc);
    return SLE_OK;
}

SLE_API void SLE_CALL sle_ExServerDestroy(SLE_ExServer* s) { delete s; }

SLE_API SLE_StatusCode SLE_CALL sle_ExServerAddGrid(SLE_ExServer* s, int32_t n_bus, const int32_t* bus_type,
                                                    const SLE_Real* v_setpoint, int32_t n_branch, const int32_t* from,
                                                    const int32_t* to, const SLE_Real* r, const SLE_Real* x,
                                                    const SLE_Real* b, const SLE_Real* tap, const SLE_Real* shift,
                                                    const int32_t* status, int32_t n_meas, const int32_t* mtype,
                                                    const int32_t* mloc, const int32_t* mend, const SLE_Real* sigma,
                                                    const SLE_Real* z, int32_t* grid_id) {
    if (!s) return SLE_ERROR_INVALID_HANDLE;
    return server_rc(s, s->srv.add_grid(n_bus, bus_type, v_setpoint, n_branch, from, to, r, x, b, tap, shift, status,
                                        n_meas, mtype, mloc, mend, sigma, z, grid_id));
}

SLE_API SLE_StatusCode SLE_CALL sle_ExServerStart(SLE_ExServer* s) {
    if (!s) return SLE_ERROR_INVALID_HANDLE;
    return server_rc(s, s->srv.start());
}

SLE_API SLE_StatusCode SLE_CALL sle_ExServerSubmit(SLE_ExServer* s, int32_t grid, const SLE_Real* values, int32_t count,
                                                   int32_t branch, int32_t closed, int64_t* ticket) {
    if (!s) return SLE_ERROR_INVALID_HANDLE;
    return server_rc(s, s->srv.submit(grid, values, count, branch, closed, ticket));
}

SLE_API SLE_StatusCode SLE_CALL sle_ExServerSubmitEx(SLE_ExServer* s, int32_t grid, const SLE_Real* values,
                                                     int32_t count, int32_t branch, int32_t closed, SLE_Real* v_out,
                                                     SLE_Real* theta_out, int64_t* ticket) {
    if (!s) return SLE_ERROR_INVALID_HANDLE;
    return server_rc(s, s->srv.submit(grid, values, count, branch, closed, ticket, v_out, theta_out));
}

SLE_API int32_t SLE_CALL sle_ExServerWait(SLE_ExServer* s, int64_t ticket, double timeout_ms, SLE_ExServeResult* res) {
    if (!s) return SLE_ERROR_INVALID_HANDLE;
    sle_gb300::ServeResult r;
    const int32_t done = s->srv.wait(ticket, timeout_ms, &r);
    if (done == 1 && res) {
        res->status = r.status;
        res->iterations = r.iterations;
        res->max_mismatch = r.max_mismatch;
        res->objective = r.objective;
        res->admitted = r.admitted;
        res->batch_size = r.batch_size;
        res->t_submit_ns = r.t_submit_ns;
        res->t_start_ns = r.t_start_ns;
        res->t_done_ns = r.t_done_ns;
    }
    return done;
}

SLE_API SLE_StatusCode SLE_CALL sle_ExServerGetState(SLE_ExServer* s, int32_t grid, SLE_Real* v, SLE_Real* theta) {
    if (!s) return SLE_ERROR_INVALID_HANDLE;
    return server_rc(s, s->srv.get_state(grid, v, theta));
}

SLE_API SLE_StatusCode SLE_CALL sle_ExServerGetStats(SLE_ExServer* s, SLE_ExServerStats* out) {
    if (!s || !out) return SLE_ERROR_INVALID_ARGUMENT;
    const sle_gb300::ServeStats st = s->srv.stats();
    out->submitted = st.submitted;
    out->completed = st.completed;
    out->rejected = st.rejected;
    out->passes = st.passes;
    out->grid_solves = st.grid_solves;
    out->units = st.units;
    out->admitted_units = st.admitted_units;
    out->grids = st.grids;
    out->pad = 0;
    out->device_bytes = st.device_bytes;
    out->budget_bytes = st.budget_bytes;
    out->admissions = st.admissions;
    out->evictions = st.evictions;
    out->resident_units = st.resident_units;
    out->pad2 = 0;
    return SLE_OK;
}

SLE_API const char* SLE_CALL sle_ExServerLastError(SLE_ExServer* s) {
    if (!s) return "invalid server";
    s->err = s->srv.last_error;
    return s->err.c_str();
}

static SLE_StatusCode batch_rc(SLE_Handle handle, int32_t rc) {
    if (rc == 0) return SLE_OK;
    const std::string& msg = E(handle)->last_error;
    if (rc == -4) return fail(SLE_ERROR_INVALID_ARGUMENT, msg);
    if (rc == -11) return fail(SLE_ERROR_ELEMENT_NOT_FOUND, msg);
    if (rc == -5) return fail(SLE_ERROR_MODEL_INCOMPLETE, msg);
    return fail(SLE_ERROR_CUDA_FAILURE, msg);
}

SLE_API SLE_StatusCode SLE_CALL sle_ExBatchAddGrid(SLE_Handle handle, int32_t n_bus, const int32_t* bus_type,
                                                   const SLE_Real* v_setpoint, int32_t n_branch, const int32_t* from,
                                                   const int32_t* to, const SLE_Real* r, const SLE_Real* x,
                                                   const SLE_Real* b, const SLE_Real* tap, const SLE_Real* shift,
                                                   const int32_t* status, int32_t n_meas, const int32_t* mtype,
                                                   const int32_t* mloc, const int32_t* mend, const SLE_Real* sigma,
                                                   const SLE_Real* z, int32_t* grid_id) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    if (bus_type)
        for (int32_t i = 0; i < n_bus; ++i)
            if (bus_type[i] < 0 || bus_type[i] > 2) return fail(SLE_ERROR_INVALID_ARGUMENT, "invalid bus type");
    return batch_rc(handle, E(handle)->batch_add_grid(n_bus, bus_type, v_setpoint, n_branch, from, to, r, x, b, tap,
                                                      shift, status, n_meas, mtype, mloc, mend, sigma, z, grid_id));
}

SLE_API int32_t SLE_CALL sle_ExBatchGridCount(SLE_Handle handle) {
    return handle ? static_cast<int32_t>(E(handle)->grids().size()) : 0;
}

SLE_API SLE_StatusCode SLE_CALL sle_ExBatchUpdateTelemetry(SLE_Handle handle, int32_t grid, const SLE_Real* values,
                                                           int32_t count) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    return batch_rc(handle, E(handle)->batch_set_telemetry(grid, values, count));
}

SLE_API SLE_StatusCode SLE_CALL sle_ExBatchSolve(SLE_Handle handle, int32_t n, const int32_t* grids,
                                                 const uint8_t* flat_start, int32_t max_iterations, double tolerance,
                                                 int32_t robust, double huber_gamma, SLE_ExGridResult* results) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    if (n < 0 || (n > 0 && !grids) || max_iterations < 1 || !(tolerance > 0.0))
        return fail(SLE_ERROR_INVALID_ARGUMENT, "invalid batch solve arguments");
    sle_gb300::SolveRequest rq;
    rq.mode = sle_gb300::Mode::PRECISION;
    rq.max_iterations = max_iterations;
    rq.tolerance = tolerance;
    rq.robust = robust;
    rq.huber_gamma = huber_gamma;
    std::vector<sle_gb300::Engine::GridResult> out(static_cast<size_t>(n));
    const int32_t rc = E(handle)->batch_solve(n, grids, flat_start, rq, out.data());
    if (rc) return batch_rc(handle, rc);
    if (results)
        for (int32_t i = 0; i < n; ++i) {
            results[i].status = out[i].status;
            results[i].iterations = out[i].iterations;
            results[i].max_mismatch = out[i].max_mismatch;
            results[i].objective = out[i].objective;
        }
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_ExBatchGetState(SLE_Handle handle, int32_t grid, SLE_Real* v, SLE_Real* theta) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    return batch_rc(handle, E(handle)->batch_get_state(grid, v, theta));
}

SLE_API SLE_StatusCode SLE_CALL sle_ExBatchSetBranchStatus(SLE_Handle handle, int32_t grid, int32_t branch,
                                                           int32_t closed) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    return batch_rc(handle, E(handle)->batch_set_branch_status(grid, branch, closed));
}

SLE_API SLE_StatusCode SLE_CALL sle_ExSetOption(SLE_Handle handle, const char* key, double value) {
    if (!handle || !key) return SLE_ERROR_INVALID_ARGUMENT;
    auto& c = E(handle)->cfg;
    const std::string k = key;
    if (k == "exact_jacobian") c.exact_jacobian = value != 0.0;
    else if (k == "gain_policy") c.gain_policy = static_cast<int32_t>(value);
    else if (k == "ordering") { c.ordering = static_cast<int32_t>(value); E(handle)->model.structure_dirty = true; }
    else if (k == "use_double_precision") {
        c.use_double_precision = value != 0.0;
        E(handle)->model.structure_dirty = true;
    } else if (k == "refine_steps") c.refine_steps = static_cast<int32_t>(value);
    else if (k == "big_front_flops") { c.big_front_flops = value; E(handle)->model.structure_dirty = true; }
    else if (k == "dataflow") { c.dataflow = value != 0.0 ? 1 : 0; E(handle)->model.structure_dirty = true; }
    else if (k == "flow_small_f") { c.flow_small_f = static_cast<int32_t>(value); E(handle)->model.structure_dirty = true; }
    else if (k == "warp_fronts") { c.warp_fronts = value < 0.0 ? -1 : (value != 0.0 ? 1 : 0); E(handle)->model.structure_dirty = true; }
    else if (k == "gain_accumulate") {
        if (value != 32.0 && value != 64.0) return fail(SLE_ERROR_INVALID_ARGUMENT, "gain_accumulate is 32 or 64");
        c.gain_acc32 = value == 32.0 ? 1 : 0;
        E(handle)->model.structure_dirty = true;  // taken at the next upload
    } else if (k == "huber_stall") {
        if (!(value >= 0.0 && value < 1.0)) return fail(SLE_ERROR_INVALID_ARGUMENT, "huber_stall must be in [0, 1)");
        c.huber_stall = value;
    } else if (k == "eval_pair_rows") {
        if (!(value >= 0.0 && value <= 2.0e9)) return fail(SLE_ERROR_INVALID_ARGUMENT, "eval_pair_rows must be >= 0");
        c.eval_pair_rows = static_cast<int32_t>(value);
        E(handle)->model.structure_dirty = true;  // taken at the next upload
    } else if (k == "tile_flow") {
        c.tile_flow = value != 0.0 ? 1 : 0;
        E(handle)->model.structure_dirty = true;  // taken at the next upload
    } else if (k == "device_loop") {
        c.device_loop = value != 0.0 ? 1 : 0;
    } else if (k == "spin_limit" || k == "hold_front") {
        if (k == "spin_limit") {
            if (!(value >= 1.0 && value <= 9.0e15)) return fail(SLE_ERROR_INVALID_ARGUMENT, "spin_limit must be >= 1");
            c.spin_limit = static_cast<long long>(value);
        } else {
            c.hold_front = value < 0.0 ? -1 : static_cast<int32_t>(value);
        }
        E(handle)->apply_wait_options();
    } else return fail(SLE_ERROR_INVALID_ARGUMENT, "unknown option");
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_ExGetScheduleInfo(SLE_Handle handle, SLE_ExScheduleInfo* info) {
    if (!handle || !info) return SLE_ERROR_INVALID_ARGUMENT;
    sle_gb300::Engine::ScheduleInfo si;
    if (E(handle)->schedule_info(si) != 0) return fail(SLE_ERROR_MODEL_INCOMPLETE, E(handle)->last_error);
    std::memset(info, 0, sizeof(*info));
    info->n_warp = si.n_warp;
    info->n_phase_a = si.n_phase_a;
    info->n_phase_b = si.n_phase_b;
    info->n_sync = si.n_sync;
    info->warp_ready = si.warp_ready;
    info->a_ready = si.a_ready;
    info->b_ready = si.b_ready;
    info->up_ready = si.up_ready;
    info->down_n = si.down_n;
    info->down_warp_n = si.down_warp_n;
    info->sync_levels = si.sync_levels;
    info->panel_steps = si.panel_steps;
    info->by_depth = si.by_depth;
    info->tile_tasks = si.tile_tasks;
    info->launches_by_height = si.launches_by_height;
    info->launches_by_depth = si.launches_by_depth;
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_ExGetPlanInfo(SLE_Handle handle, SLE_ExPlanInfo* info) {
    if (!handle || !info) return SLE_ERROR_INVALID_ARGUMENT;
    Engine* e = E(handle);
    if (!e->analyzed() || e->model.structure_dirty) {
        if (e->analyze() != 0) return fail(SLE_ERROR_MODEL_INCOMPLETE, e->last_error);
    }
    const auto& P = e->plan();
    std::memset(info, 0, sizeof(*info));
    info->n_bus = P.n_bus;
    info->n_state = P.n_state;
    info->n_meas = P.n_meas;
    info->nnz_ybus = static_cast<int32_t>(P.y_col.size());
    info->nnz_h = static_cast<int64_t>(P.h_col.size());
    info->n_super = P.n_super;
    info->n_levels = P.n_levels;
    info->max_front = P.max_front;
    info->nnz_l = P.nnz_l;
    info->lx_size = P.lx_size;
    info->u_size = P.u_size;
    info->n_gain_targets = static_cast<int64_t>(P.tgt_local.size());
    info->n_gain_pairs = static_cast<int64_t>(P.pair_a.size());
    info->factor_flops = P.flops;
    info->device_bytes = e->device_bytes();
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_ExGetYbus(SLE_Handle handle, int32_t* row_ptr, int32_t* col, SLE_Real* g,
                                              SLE_Real* b) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    Engine* e = E(handle);
    if (!e->analyzed() || e->model.structure_dirty) {
        if (e->analyze() != 0) return fail(SLE_ERROR_MODEL_INCOMPLETE, e->last_error);
    }
    const auto& P = e->plan();
    if (row_ptr) std::memcpy(row_ptr, P.y_ptr.data(), sizeof(int32_t) * P.y_ptr.size());
    if (col) std::memcpy(col, P.y_col.data(), sizeof(int32_t) * P.y_col.size());
    if (g || b) {
        if (!e->uploaded()) return fail(SLE_ERROR_NOT_INITIALIZED, "model not uploaded");
        std::vector<double> gv, bv;
        if (e->export_ybus(gv, bv) != 0) return fail(SLE_ERROR_CUDA_FAILURE, e->last_error);
        if (g) std::memcpy(g, gv.data(), sizeof(double) * gv.size());
        if (b) std::memcpy(b, bv.data(), sizeof(double) * bv.size());
    }
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_ExEvaluateAt(SLE_Handle handle, const SLE_Real* v, const SLE_Real* theta,
                                                 int32_t exact_jacobian) {
    if (!handle || !v || !theta) return SLE_ERROR_INVALID_ARGUMENT;
    if (E(handle)->evaluate_at(v, theta, exact_jacobian) != 0) return fail(SLE_ERROR_CUDA_FAILURE, E(handle)->last_error);
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_ExGetJacobian(SLE_Handle handle, int32_t* row_ptr, int32_t* col, SLE_Real* val,
                                                  SLE_Real* hx, SLE_Real* rhs) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    Engine* e = E(handle);
    if (!e->analyzed() || e->model.structure_dirty) {
        if (e->analyze() != 0) return fail(SLE_ERROR_MODEL_INCOMPLETE, e->last_error);
    }
    const auto& P = e->plan();
    if (row_ptr) std::memcpy(row_ptr, P.h_ptr.data(), sizeof(int32_t) * P.h_ptr.size());
    if (col) std::memcpy(col, P.h_col.data(), sizeof(int32_t) * P.h_col.size());
    if (val || hx || rhs) {
        if (!e->uploaded()) return fail(SLE_ERROR_NOT_INITIALIZED, "model not uploaded");
        if (e->export_eval(val, hx, rhs) != 0) return fail(SLE_ERROR_CUDA_FAILURE, e->last_error);
    }
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_ExGetGain(SLE_Handle handle, int32_t* rows, int32_t* cols, SLE_Real* vals) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    std::vector<int32_t> r, c;
    std::vector<double> v;
    if (E(handle)->export_gain(r, c, v) != 0) return fail(SLE_ERROR_CUDA_FAILURE, E(handle)->last_error);
    if (rows) std::memcpy(rows, r.data(), sizeof(int32_t) * r.size());
    if (cols) std::memcpy(cols, c.data(), sizeof(int32_t) * c.size());
    if (vals) std::memcpy(vals, v.data(), sizeof(double) * v.size());
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_ExFactorSolve(SLE_Handle handle, const SLE_Real* rhs, SLE_Real* x) {
    if (!handle || !rhs || !x) return SLE_ERROR_INVALID_ARGUMENT;
    const int32_t rc = E(handle)->factor_and_solve(rhs, x);
    if (rc == -7) return fail(SLE_ERROR_SINGULAR_MATRIX, "gain matrix is not positive definite");
    if (rc) return fail(SLE_ERROR_CUDA_FAILURE, E(handle)->last_error);
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_ExFactorSolveNoAlloc(SLE_Handle handle, const SLE_Real* rhs, SLE_Real* x) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    if (!rhs || !x) return SLE_ERROR_INVALID_ARGUMENT;
    const int32_t rc = E(handle)->factor_and_solve_noalloc(rhs, x);
    if (rc == -7) return fail(SLE_ERROR_SINGULAR_MATRIX, "gain matrix is not positive definite");
    if (rc == -11) return fail(SLE_ERROR_INVALID_ARGUMENT, E(handle)->last_error);
    if (rc) return fail(SLE_ERROR_CUDA_FAILURE, E(handle)->last_error);
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_ExGetSymbolic(SLE_Handle handle, int32_t* bus_perm, int32_t* state_of_ps,
                                                  int32_t* sn_c0, int32_t* sn_parent, int64_t* sn_rows_off,
                                                  int32_t* sn_rows) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    Engine* e = E(handle);
    if (!e->analyzed() || e->model.structure_dirty) {
        if (e->analyze() != 0) return fail(SLE_ERROR_MODEL_INCOMPLETE, e->last_error);
    }
    const auto& P = e->plan();
    if (bus_perm) std::memcpy(bus_perm, P.bus_perm.data(), sizeof(int32_t) * P.bus_perm.size());
    if (state_of_ps) std::memcpy(state_of_ps, P.state_of_ps.data(), sizeof(int32_t) * P.state_of_ps.size());
    if (sn_c0) std::memcpy(sn_c0, P.sn_c0.data(), sizeof(int32_t) * P.sn_c0.size());
    if (sn_parent) std::memcpy(sn_parent, P.sn_parent.data(), sizeof(int32_t) * P.sn_parent.size());
    if (sn_rows_off) std::memcpy(sn_rows_off, P.sn_rows_off.data(), sizeof(int64_t) * P.sn_rows_off.size());
    if (sn_rows) std::memcpy(sn_rows, P.sn_rows.data(), sizeof(int32_t) * P.sn_rows.size());
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_ExStageTelemetry(SLE_Handle handle, const SLE_Real* values, int32_t count,
                                                     int32_t slot) {
    if (!handle || !values) return SLE_ERROR_INVALID_ARGUMENT;
    const int32_t rc = E(handle)->stage_telemetry(values, count, slot);
    if (rc == -4) return fail(SLE_ERROR_INVALID_ARGUMENT, E(handle)->last_error);
    if (rc) return fail(SLE_ERROR_CUDA_FAILURE, E(handle)->last_error);
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_ExUseTelemetry(SLE_Handle handle, int32_t slot) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    const int32_t rc = E(handle)->use_telemetry(slot);
    if (rc == -4) return fail(SLE_ERROR_INVALID_ARGUMENT, E(handle)->last_error);
    if (rc) return fail(SLE_ERROR_CUDA_FAILURE, E(handle)->last_error);
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_ExFlushL2(SLE_Handle handle, size_t bytes) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    if (E(handle)->flush_l2(bytes) != 0) return fail(SLE_ERROR_CUDA_FAILURE, E(handle)->last_error);
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_ExTimer(SLE_Handle handle, int32_t op, double* elapsed_ms) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    if (E(handle)->timer(op, elapsed_ms) != 0) return fail(SLE_ERROR_CUDA_FAILURE, E(handle)->last_error);
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_ExGetStats(SLE_Handle handle, SLE_ExStats* st) {
    if (!handle || !st) return SLE_ERROR_INVALID_ARGUMENT;
    const auto& s = E(handle)->stats;
    for (int i = 0; i < 6; ++i) {
        st->launches[i] = s.launches[i];
        st->ms[i] = s.ms[i];
        st->calls[i] = s.calls[i];
    }
    st->iterations = s.iterations;
    st->solves = s.solves;
    st->total_launches = sle_gb300::g_kernel_launches.load();
    st->analyses = s.analyses;
    st->uploads = s.uploads;
    st->branch_edits = s.branch_edits;
    st->step_waits = s.step_waits;
    st->analysis_ms = s.analysis_ms;
    st->schedule_ms = s.schedule_ms;
    st->upload_ms = s.upload_ms;
    st->capture_ms = s.capture_ms;
    return SLE_OK;
}

SLE_API SLE_StatusCode SLE_CALL sle_ExResetStats(SLE_Handle handle) {
    if (!handle) return SLE_ERROR_INVALID_HANDLE;
    E(handle)->stats = sle_gb300::StageStats();
    return SLE_OK;
}

}  // extern "C"
