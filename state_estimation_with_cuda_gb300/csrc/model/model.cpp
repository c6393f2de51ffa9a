#include "model.h"

#include <algorithm>

namespace sle_gb300 {

namespace {
inline bool is_bus_meas(int32_t t) { return t == 0 || t == 1 || t == 2 || t == 3 || t == 7 || t == 8; }
}  // namespace

void Model::ensure_names() {
    if (names_ready) return;
    bus_map.clear();
    br_map.clear();
    m_map.clear();
    bus_id.resize(n_bus());
    for (int32_t i = 0; i < n_bus(); ++i) {
        if (bus_id[i].empty()) bus_id[i] = "BUS" + std::to_string(i);
        bus_map[bus_id[i]] = i;
    }
    br_id.resize(n_branch());
    br_sd.resize(n_branch());
    for (int32_t k = 0; k < n_branch(); ++k) {
        if (br_id[k].empty()) br_id[k] = "BR" + std::to_string(k);
        br_map[br_id[k]] = k;
    }
    m_id.resize(n_meas());
    for (int32_t q = 0; q < n_meas(); ++q) {
        if (m_id[q].empty()) m_id[q] = "M" + std::to_string(q);
        m_map[m_id[q]] = q;
    }
    names_ready = true;
}

int32_t Model::find_bus(const std::string& id) {
    ensure_names();
    auto it = bus_map.find(id);
    return it == bus_map.end() ? -1 : it->second;
}
int32_t Model::find_branch(const std::string& id) {
    ensure_names();
    auto it = br_map.find(id);
    return it == br_map.end() ? -1 : it->second;
}
int32_t Model::find_meas(const std::string& id) {
    ensure_names();
    auto it = m_map.find(id);
    return it == m_map.end() ? -1 : it->second;
}
int32_t Model::find_switch(const std::string& id) {
    auto it = sd_map.find(id);
    return it == sd_map.end() ? -1 : it->second;
}
int32_t Model::find_meter(const std::string& id) {
    auto it = meter_map.find(id);
    return it == meter_map.end() ? -1 : it->second;
}

int32_t Model::add_bus(const std::string& id, double kv, int32_t type, double vset, double p, double q) {
    if (type < 0 || type > 2) return -4;
    if (find_bus(id) >= 0) return -12;
    const int32_t idx = n_bus();
    bus_id.push_back(id);
    bus_kv.push_back(kv);
    bus_type.push_back(type);
    bus_vset.push_back(vset);
    bus_p.push_back(p);
    bus_q.push_back(q);
    bus_v.push_back(vset);  // network_model.cu:76-83: state starts at the setpoint
    bus_th.push_back(0.0);
    bus_map[id] = idx;
    if (type == 2) slack = idx;
    structure_dirty = true;
    return idx;
}

int32_t Model::add_branch(const std::string& id, const std::string& from, const std::string& to, double r, double x,
                          double b, double g, double tap, double shift, int32_t xfmr, const std::string& sd) {
    if (find_branch(id) >= 0) return -12;
    const int32_t f = find_bus(from), t = find_bus(to);
    if (f < 0 || t < 0) return -11;
    const int32_t idx = n_branch();
    br_id.push_back(id);
    br_sd.push_back(sd);
    br_from.push_back(f);
    br_to.push_back(t);
    br_xfmr.push_back(xfmr);
    br_r.push_back(r);
    br_x.push_back(x);
    br_b.push_back(b);
    br_g.push_back(g);
    br_tap.push_back(tap);
    br_shift.push_back(shift);
    br_closed.push_back(1);
    br_map[id] = idx;
    structure_dirty = true;
    return idx;
}

int32_t Model::add_measurement(const std::string& id, int32_t type, const std::string& loc, int32_t end, double sigma,
                               double pt, double ct, int32_t pseudo) {
    if (type < 0 || type > 8) return -4;
    if (find_meas(id) >= 0) return -12;
    const int32_t l = is_bus_meas(type) ? find_bus(loc) : find_branch(loc);
    if (l < 0) return -11;
    const int32_t idx = n_meas();
    m_id.push_back(id);
    m_type.push_back(type);
    m_loc.push_back(l);
    m_end.push_back(end ? 1 : 0);
    m_pseudo.push_back(pseudo);
    m_sigma.push_back(sigma);
    m_pt.push_back(pt);
    m_ct.push_back(ct);
    m_value.push_back(0.0);
    const double s = std::max(sigma, kRealEps);
    m_w.push_back(1.0 / (s * s));
    m_active.push_back(1);
    m_est.push_back(0.0);
    m_res.push_back(0.0);
    m_map[id] = idx;
    structure_dirty = true;
    return idx;
}

int32_t Model::add_switch(const std::string& id, const std::string& branch, int32_t closed) {
    if (find_switch(id) >= 0) return -12;
    const int32_t k = find_branch(branch);
    if (k < 0) return -11;
    const int32_t idx = static_cast<int32_t>(sd_id.size());
    sd_id.push_back(id);
    sd_branch.push_back(k);
    sd_closed.push_back(closed ? 1 : 0);
    sd_map[id] = idx;
    if (!closed) {
        br_closed[k] = 0;
        structure_dirty = true;
    }
    return idx;
}

int32_t Model::channel_meas(const Meter& m, const std::string& c) {
    if (c == "V" || c == "kV" || c == "voltage") return m.m_v;
    if (c == "kW" || c == "MW" || c == "P" || c == "power") return m.m_p;
    if (c == "kVAR" || c == "MVAR" || c == "Q" || c == "reactive") return m.m_q;
    if (c == "A" || c == "kA" || c == "I" || c == "current") return m.m_i;
    return -1;
}

int32_t Model::add_meter(const Meter& in, const std::string& bus_name, const std::string& branch_name) {
    if (in.type < 0 || in.type > 3) return -4;
    if (find_meter(in.id) >= 0) return -12;
    if (find_bus(bus_name) < 0) return -11;
    if (in.type != 0 && find_branch(branch_name) < 0) return -11;
    Meter m = in;
    m.bus = find_bus(bus_name);
    m.branch = in.type != 0 ? find_branch(branch_name) : -1;
    auto add = [&](const char* suffix, int32_t type, const std::string& loc, double sigma) {
        return add_measurement(m.id + suffix, type, loc, m.end, sigma, m.pt, type == 0 ? 1.0 : m.ct, 0);
    };
    // network_model.cu:339-377: ".V", ".kW", ".kVAR", ".A" in that order
    if (m.type == 0) {
        m.m_v = add(".V", 0, bus_name, m.sigma_v);
    } else if (m.type == 1) {
        m.m_v = add(".V", 0, bus_name, m.sigma_v);
        m.m_p = add(".kW", 4, branch_name, m.sigma_p);
        m.m_q = add(".kVAR", 5, branch_name, m.sigma_p);
        m.m_i = add(".A", 6, branch_name, m.sigma_i);
    } else if (m.type == 2) {
        m.m_i = add(".A", 6, branch_name, m.sigma_i);
    } else {
        m.m_p = add(".kW", 4, branch_name, m.sigma_p);
        m.m_q = add(".kVAR", 5, branch_name, m.sigma_p);
    }
    const int32_t idx = static_cast<int32_t>(meters.size());
    meters.push_back(m);
    meter_map[m.id] = idx;
    structure_dirty = true;
    return idx;
}

namespace {
template <typename T>
void compact(std::vector<T>& v, const std::vector<char>& keep) {
    size_t o = 0;
    for (size_t i = 0; i < v.size(); ++i)
        if (keep[i]) v[o++] = v[i];
    v.resize(o);
}
}  // namespace

int32_t Model::remove_branch(const std::string& id) {
    const int32_t k = find_branch(id);
    if (k < 0) return -11;
    std::vector<char> keep_br(n_branch(), 1), keep_m(n_meas(), 1);
    keep_br[k] = 0;
    for (int32_t q = 0; q < n_meas(); ++q)
        if (!is_bus_meas(m_type[q]) && m_loc[q] == k) keep_m[q] = 0;
    // re-index
    std::vector<int32_t> new_br(n_branch(), -1), new_m(n_meas(), -1);
    for (int32_t i = 0, o = 0; i < n_branch(); ++i) if (keep_br[i]) new_br[i] = o++;
    for (int32_t i = 0, o = 0; i < n_meas(); ++i) if (keep_m[i]) new_m[i] = o++;
    for (int32_t q = 0; q < n_meas(); ++q)
        if (keep_m[q] && !is_bus_meas(m_type[q])) m_loc[q] = new_br[m_loc[q]];
    for (auto* v : {&br_id, &br_sd}) compact(*v, keep_br);
    for (auto* v : {&br_from, &br_to, &br_xfmr}) compact(*v, keep_br);
    for (auto* v : {&br_r, &br_x, &br_b, &br_g, &br_tap, &br_shift}) compact(*v, keep_br);
    compact(br_closed, keep_br);
    compact(m_id, keep_m);
    for (auto* v : {&m_type, &m_loc, &m_end, &m_pseudo}) compact(*v, keep_m);
    for (auto* v : {&m_sigma, &m_pt, &m_ct, &m_value, &m_w, &m_est, &m_res}) compact(*v, keep_m);
    compact(m_active, keep_m);
    // switches on the removed branch go away; others re-index
    std::vector<char> keep_sd(sd_id.size(), 1);
    for (size_t s = 0; s < sd_id.size(); ++s) {
        if (sd_branch[s] == k) keep_sd[s] = 0;
        else sd_branch[s] = new_br[sd_branch[s]];
    }
    compact(sd_id, keep_sd);
    compact(sd_branch, keep_sd);
    compact(sd_closed, keep_sd);
    sd_map.clear();
    for (size_t s = 0; s < sd_id.size(); ++s) sd_map[sd_id[s]] = static_cast<int32_t>(s);
    for (auto& m : meters) {
        if (m.branch == k) m.branch = -1;
        else if (m.branch >= 0) m.branch = new_br[m.branch];
        for (int32_t* mi : {&m.m_v, &m.m_p, &m.m_q, &m.m_i})
            if (*mi >= 0) *mi = new_m[*mi];
    }
    names_ready = false;
    ensure_names();
    structure_dirty = true;
    return 0;
}

int32_t Model::remove_bus(const std::string& id) {
    const int32_t b = find_bus(id);
    if (b < 0) return -11;
    // drop branches touching the bus first
    for (;;) {
        int32_t k = -1;
        for (int32_t x = 0; x < n_branch(); ++x)
            if (br_from[x] == b || br_to[x] == b) { k = x; break; }
        if (k < 0) break;
        ensure_names();
        remove_branch(br_id[k]);
    }
    std::vector<char> keep_b(n_bus(), 1), keep_m(n_meas(), 1);
    keep_b[b] = 0;
    for (int32_t q = 0; q < n_meas(); ++q)
        if (is_bus_meas(m_type[q]) && m_loc[q] == b) keep_m[q] = 0;
    std::vector<int32_t> new_b(n_bus(), -1), new_m(n_meas(), -1);
    for (int32_t i = 0, o = 0; i < n_bus(); ++i) if (keep_b[i]) new_b[i] = o++;
    for (int32_t i = 0, o = 0; i < n_meas(); ++i) if (keep_m[i]) new_m[i] = o++;
    for (int32_t q = 0; q < n_meas(); ++q)
        if (keep_m[q] && is_bus_meas(m_type[q])) m_loc[q] = new_b[m_loc[q]];
    for (int32_t k = 0; k < n_branch(); ++k) {
        br_from[k] = new_b[br_from[k]];
        br_to[k] = new_b[br_to[k]];
    }
    compact(bus_id, keep_b);
    for (auto* v : {&bus_kv, &bus_vset, &bus_p, &bus_q, &bus_v, &bus_th}) compact(*v, keep_b);
    compact(bus_type, keep_b);
    compact(m_id, keep_m);
    for (auto* v : {&m_type, &m_loc, &m_end, &m_pseudo}) compact(*v, keep_m);
    for (auto* v : {&m_sigma, &m_pt, &m_ct, &m_value, &m_w, &m_est, &m_res}) compact(*v, keep_m);
    compact(m_active, keep_m);
    std::vector<Meter> kept;
    for (auto& m : meters) {
        if (m.bus == b) continue;
        m.bus = new_b[m.bus];
        for (int32_t* mi : {&m.m_v, &m.m_p, &m.m_q, &m.m_i})
            if (*mi >= 0) *mi = new_m[*mi];
        kept.push_back(m);
    }
    meters.swap(kept);
    meter_map.clear();
    for (size_t i = 0; i < meters.size(); ++i) meter_map[meters[i].id] = static_cast<int32_t>(i);
    slack = -1;
    for (int32_t i = 0; i < n_bus(); ++i)
        if (bus_type[i] == 2) slack = i;
    names_ready = false;
    ensure_names();
    structure_dirty = true;
    return 0;
}

void Model::load_soa(int32_t nb, const int32_t* btype, const double* vset, int32_t nbr, const int32_t* from,
                     const int32_t* to, const double* r, const double* x, const double* b, const double* tap,
                     const double* shift, const int32_t* status, int32_t nm, const int32_t* mtype,
                     const int32_t* mloc, const int32_t* mend, const double* sigma, const double* z) {
    clear();
    bus_type.assign(btype, btype + nb);
    bus_vset.assign(vset, vset + nb);
    bus_kv.assign(nb, 1.0);
    bus_p.assign(nb, 0.0);
    bus_q.assign(nb, 0.0);
    bus_v.assign(vset, vset + nb);
    bus_th.assign(nb, 0.0);
    bus_id.clear();  // names: default ones, made by ensure_names() at the first lookup
    for (int32_t i = 0; i < nb; ++i)
        if (btype[i] == 2) slack = i;
    br_from.assign(from, from + nbr);
    br_to.assign(to, to + nbr);
    br_r.assign(r, r + nbr);
    br_x.assign(x, x + nbr);
    br_b.assign(b, b + nbr);
    br_g.assign(nbr, 0.0);
    br_tap.assign(tap, tap + nbr);
    br_shift.assign(shift, shift + nbr);
    br_xfmr.assign(nbr, 0);
    br_closed.resize(nbr);
    for (int32_t k = 0; k < nbr; ++k) br_closed[k] = status ? (status[k] ? 1 : 0) : 1;
    br_id.clear();
    br_sd.clear();
    m_type.assign(mtype, mtype + nm);
    m_loc.assign(mloc, mloc + nm);
    m_end.assign(mend, mend + nm);
    m_pseudo.assign(nm, 0);
    m_sigma.assign(sigma, sigma + nm);
    m_pt.assign(nm, 1.0);
    m_ct.assign(nm, 1.0);
    m_value.assign(z, z + nm);
    m_w.resize(nm);
    for (int32_t q = 0; q < nm; ++q) {
        const double s = std::max(sigma[q], kRealEps);
        m_w[q] = 1.0 / (s * s);
    }
    m_active.assign(nm, 1);
    m_est.assign(nm, 0.0);
    m_res.assign(nm, 0.0);
    m_id.clear();
    names_ready = false;
    structure_dirty = true;
}

void Model::append_soa(int32_t nb, const int32_t* btype, const double* vset, int32_t nbr, const int32_t* from,
                       const int32_t* to, const double* r, const double* x, const double* b, const double* tap,
                       const double* shift, const int32_t* status, int32_t nm, const int32_t* mtype,
                       const int32_t* mloc, const int32_t* mend, const double* sigma, const double* z) {
    const int32_t b0 = n_bus(), k0 = n_branch();
    for (int32_t i = 0; i < nb; ++i) {
        bus_type.push_back(btype[i]);
        bus_vset.push_back(vset[i]);
        bus_kv.push_back(1.0);
        bus_p.push_back(0.0);
        bus_q.push_back(0.0);
        bus_v.push_back(vset[i]);
        bus_th.push_back(0.0);
        bus_id.emplace_back();
        if (btype[i] == 2 && slack < 0) slack = b0 + i;
    }
    for (int32_t k = 0; k < nbr; ++k) {
        br_from.push_back(from[k] + b0);
        br_to.push_back(to[k] + b0);
        br_r.push_back(r[k]);
        br_x.push_back(x[k]);
        br_b.push_back(b[k]);
        br_g.push_back(0.0);
        br_tap.push_back(tap[k]);
        br_shift.push_back(shift[k]);
        br_xfmr.push_back(0);
        br_closed.push_back(status ? (status[k] ? 1 : 0) : 1);
        br_id.emplace_back();
        br_sd.emplace_back();
    }
    for (int32_t q = 0; q < nm; ++q) {
        const int32_t ty = mtype[q];
        const bool on_branch = (ty == 4 || ty == 5 || ty == 6);
        m_type.push_back(ty);
        m_loc.push_back(mloc[q] + (on_branch ? k0 : b0));
        m_end.push_back(mend[q]);
        m_pseudo.push_back(0);
        m_sigma.push_back(sigma[q]);
        m_pt.push_back(1.0);
        m_ct.push_back(1.0);
        m_value.push_back(z[q]);
        const double s = std::max(sigma[q], kRealEps);
        m_w.push_back(1.0 / (s * s));
        m_active.push_back(1);
        m_est.push_back(0.0);
        m_res.push_back(0.0);
        m_id.emplace_back();
    }
    names_ready = false;
    structure_dirty = true;
}

void Model::clear() { *this = Model(); }

bool Model::validate(std::string& err) const {
    if (n_bus() == 0) { err = "model has no buses"; return false; }
    if (slack < 0) { err = "model has no slack bus"; return false; }
    for (int32_t k = 0; k < n_branch(); ++k) {
        if (br_from[k] < 0 || br_from[k] >= n_bus() || br_to[k] < 0 || br_to[k] >= n_bus()) {
            err = "branch references an unknown bus";
            return false;
        }
    }
    for (int32_t q = 0; q < n_meas(); ++q) {
        const int32_t lim = is_bus_meas(m_type[q]) ? n_bus() : n_branch();
        if (m_loc[q] < 0 || m_loc[q] >= lim) { err = "measurement location out of range"; return false; }
    }
    return true;
}

}  // namespace sle_gb300
