// Host-side network model: elements in insertion order with string-ID maps.
//
// Index rules follow the reference NetworkModel (network_model.cu:71-151):
// bus / branch / measurement index = insertion order; the last SLACK bus
// added becomes the slack; measurement weight = 1 / max(sigma, eps)^2;
// meters expand to measurements ".V", ".kW", ".kVAR", ".A" in that order
// (network_model.cu:312-380).  Bulk-loaded models (sle_ExLoadNetwork) carry
// no string IDs until one is asked for; synthetic IDs are then generated.
#pragma once

#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

namespace sle_gb300 {

constexpr double kRealEps = 1e-12;

struct Meter {
    std::string id;
    int32_t type = 0;
    int32_t bus = -1, branch = -1, end = 0;
    double pt = 1.0, ct = 1.0, sigma_v = 0.0, sigma_p = 0.0, sigma_i = 0.0;
    int32_t m_v = -1, m_p = -1, m_q = -1, m_i = -1;
};

struct Model {
    // Names (bus_id, br_id, br_sd, m_id) may be shorter than the element
    // arrays after a bulk load: ensure_names() sizes them and gives unnamed
    // elements their default names; every lookup calls it first.
    // buses
    std::vector<std::string> bus_id;
    std::vector<double> bus_kv, bus_vset, bus_p, bus_q;
    std::vector<int32_t> bus_type;
    std::vector<double> bus_v, bus_th;  // current state (estimate / hot start)
    int32_t slack = -1;
    // branches
    std::vector<std::string> br_id, br_sd;
    std::vector<int32_t> br_from, br_to, br_xfmr;
    std::vector<double> br_r, br_x, br_b, br_g, br_tap, br_shift;
    std::vector<uint8_t> br_closed;
    // measurements
    std::vector<std::string> m_id;
    std::vector<int32_t> m_type, m_loc, m_end, m_pseudo;
    std::vector<double> m_sigma, m_pt, m_ct, m_value, m_w;
    std::vector<uint8_t> m_active;
    std::vector<double> m_est, m_res;  // last estimate h(x) and residual
    // switching devices
    std::vector<std::string> sd_id;
    std::vector<int32_t> sd_branch;
    std::vector<uint8_t> sd_closed;
    // meters
    std::vector<Meter> meters;

    // lookup maps (built lazily for bulk-loaded models)
    std::unordered_map<std::string, int32_t> bus_map, br_map, m_map, sd_map, meter_map;
    bool names_ready = true;

    // true when the topology / parameters / measurement set changed since the
    // last upload (forces symbolic analysis + re-upload on the next solve)
    bool structure_dirty = true;
    // true when measurement values changed on the host only
    bool values_dirty = false;
    // true when branch parameters or switch states changed on the host only
    // (value edits: the uploaded pattern holds every affected branch)
    bool branch_values_dirty = false;

    int32_t n_bus() const { return static_cast<int32_t>(bus_type.size()); }
    int32_t n_branch() const { return static_cast<int32_t>(br_from.size()); }
    int32_t n_meas() const { return static_cast<int32_t>(m_type.size()); }

    void ensure_names();
    int32_t find_bus(const std::string& id);
    int32_t find_branch(const std::string& id);
    int32_t find_meas(const std::string& id);
    int32_t find_switch(const std::string& id);
    int32_t find_meter(const std::string& id);

    // Return codes: >= 0 index, -11 not found, -12 duplicate, -4 invalid.
    int32_t add_bus(const std::string& id, double kv, int32_t type, double vset, double p, double q);
    int32_t add_branch(const std::string& id, const std::string& from, const std::string& to, double r, double x,
                       double b, double g, double tap, double shift, int32_t xfmr, const std::string& sd);
    int32_t add_measurement(const std::string& id, int32_t type, const std::string& loc, int32_t end, double sigma,
                            double pt, double ct, int32_t pseudo);
    int32_t add_switch(const std::string& id, const std::string& branch, int32_t closed);
    int32_t add_meter(const Meter& m, const std::string& bus_id, const std::string& branch_id);
    int32_t remove_bus(const std::string& id);
    int32_t remove_branch(const std::string& id);

    // Meter channel -> measurement index (-1 when the meter has no such channel).
    static int32_t channel_meas(const Meter& m, const std::string& channel);

    // Bulk SoA load (no string IDs).
    void load_soa(int32_t n_bus, const int32_t* bus_type, const double* vset, int32_t n_br, const int32_t* from,
                  const int32_t* to, const double* r, const double* x, const double* b, const double* tap,
                  const double* shift, const int32_t* status, int32_t n_meas, const int32_t* mtype,
                  const int32_t* mloc, const int32_t* mend, const double* sigma, const double* z);

    // Append one more independent grid (batch mode): bus indices of branches
    // and bus-located rows are shifted by the current bus count, branch-located
    // rows (flows, currents) by the current branch count.  The first grid's
    // slack stays the model's slack.
    void append_soa(int32_t n_bus, const int32_t* bus_type, const double* vset, int32_t n_br, const int32_t* from,
                    const int32_t* to, const double* r, const double* x, const double* b, const double* tap,
                    const double* shift, const int32_t* status, int32_t n_meas, const int32_t* mtype,
                    const int32_t* mloc, const int32_t* mend, const double* sigma, const double* z);

    void clear();
    // Structural validity (reference network_model.cu:576-593).
    bool validate(std::string& err) const;
};

}  // namespace sle_gb300
