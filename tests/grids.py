"""Test grids: the reference IEEE 14-bus fixture and seeded synthetic grids."""
import json
import os
from types import SimpleNamespace

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUS_TYPES = (0, 1, 2, 3, 7, 8)


def ieee14():
    """IEEE 14-bus model + true telemetry from tests/golden/ieee14.json, as SoA
    arrays in insertion order (the index rules of sle_AddBus / AddBranch /
    AddMeasurement)."""
    with open(os.path.join(HERE, "golden", "ieee14.json")) as fh:
        d = json.load(fh)
    bid = {b["id"]: i for i, b in enumerate(d["buses"])}
    brid = {b["id"]: k for k, b in enumerate(d["branches"])}
    g = SimpleNamespace(raw=d)
    g.n_bus, g.n_branch, g.n_meas = len(d["buses"]), len(d["branches"]), len(d["measurements"])
    g.bus_type = np.array([b["type"] for b in d["buses"]], np.int32)
    g.v_setpoint = np.array([b["v_setpoint"] for b in d["buses"]])
    g.slack = int(np.where(g.bus_type == 2)[0][-1])
    g.br_from = np.array([bid[b["from"]] for b in d["branches"]], np.int32)
    g.br_to = np.array([bid[b["to"]] for b in d["branches"]], np.int32)
    g.br_r = np.array([b["r"] for b in d["branches"]])
    g.br_x = np.array([b["x"] for b in d["branches"]])
    g.br_b = np.array([b["b"] for b in d["branches"]])
    g.br_tap = np.array([b["tap"] for b in d["branches"]])
    g.br_shift = np.array([b["shift"] for b in d["branches"]])
    g.br_status = np.ones(g.n_branch, np.int32)
    g.m_type = np.array([m["type"] for m in d["measurements"]], np.int32)
    g.m_loc = np.array([bid[m["location"]] if m["type"] in BUS_TYPES else brid[m["location"]]
                        for m in d["measurements"]], np.int32)
    g.m_end = np.array([m["end"] for m in d["measurements"]], np.int32)
    g.m_sigma = np.array([m["sigma"] for m in d["measurements"]])
    g.z = np.array([d["true_telemetry"][m["id"]] for m in d["measurements"]])
    return g


def observable_ieee14():
    """The IEEE 14-bus network with the reference's fixture telemetry plus a
    P+Q injection pair at every bus, which makes the set observable."""
    g = ieee14()
    extra_t, extra_l = [], []
    for i in range(g.n_bus):
        extra_t += [2, 3]
        extra_l += [i, i]
    g.m_type = np.concatenate([g.m_type, np.array(extra_t, np.int32)])
    g.m_loc = np.concatenate([g.m_loc, np.array(extra_l, np.int32)])
    g.m_end = np.concatenate([g.m_end, np.zeros(len(extra_t), np.int32)])
    g.m_sigma = np.concatenate([g.m_sigma, np.full(len(extra_t), 0.02)])
    g.n_meas = len(g.m_type)
    g.z = np.zeros(g.n_meas)
    return g


def synthetic_state(g, seed=7):
    """A non-flat state near the grid's true operating point."""
    rng = np.random.default_rng(seed)
    v = 1.0 + 0.03 * rng.standard_normal(g.n_bus)
    th = 0.1 * rng.standard_normal(g.n_bus)
    th[g.slack] = 0.0
    return v, th


def state_index(g, bus, which):
    """State vector index of theta (which=0) or V (which=1) of a bus."""
    if which == 1:
        return g.n_bus - 1 + bus
    if bus == g.slack:
        return -1
    return bus if bus < g.slack else bus - 1


GRID_ARRAYS = ("bus_type", "v_setpoint", "br_from", "br_to", "br_r", "br_x", "br_b", "br_tap", "br_shift",
               "br_status", "m_type", "m_loc", "m_end", "m_sigma", "z")


def copy_grid(g):
    """A mutable copy of a grid's arrays (SyntheticGrid or namespace)."""
    c = SimpleNamespace(n_bus=g.n_bus, n_branch=g.n_branch, n_meas=g.n_meas, slack=g.slack)
    for k in GRID_ARRAYS:
        setattr(c, k, np.array(getattr(g, k), copy=True))
    for k in ("v_true", "theta_true"):
        if hasattr(g, k):
            setattr(c, k, np.array(getattr(g, k), copy=True))
    return c


def with_current_rows(g, n_branches, sigma=0.008, seed=5):
    """Copy of a synthetic grid with |I| rows (MEAS_I_MAG = 6) at both ends of
    `n_branches` seeded branches; their telemetry is h(x_true) from the oracle
    plus Gaussian noise of `sigma`."""
    from oracle.binding import Oracle

    c = copy_grid(g)
    rng = np.random.default_rng(seed)
    br = np.sort(rng.choice(g.n_branch, size=n_branches, replace=False)).astype(np.int32)
    c.m_type = np.concatenate([c.m_type, np.full(2 * n_branches, 6, np.int32)])
    c.m_loc = np.concatenate([c.m_loc, np.repeat(br, 2)])
    c.m_end = np.concatenate([c.m_end, np.tile(np.array([0, 1], np.int32), n_branches)])
    c.m_sigma = np.concatenate([c.m_sigma, np.full(2 * n_branches, sigma)])
    c.n_meas = len(c.m_type)
    o = Oracle(c)
    zt = np.concatenate([c.z, np.zeros(2 * n_branches)])
    hx = o.evaluate(c.v_true, c.theta_true, zt)["hx"]
    c.z = np.concatenate([c.z, hx[g.n_meas:] + sigma * rng.standard_normal(2 * n_branches)])
    o.close()
    return c


def bounded_degree_grid(n_bus, seed, max_degree=4, n_chords=None, current_rows=8):
    """A seeded grid whose buses all have at most `max_degree` branches and
    no parallel branches, so every injection row of the reference's Jacobian
    fits its fixed 10 slots (2 x 4 neighbours + 2; sparse_matrix.cu:1574-1595).
    Spanning tree (each bus joins an earlier bus with room) plus chords between
    nearby buses; parameters drawn as the synthetic workloads draw them
    (r ~ U(0.01, 0.08), x = r U(3, 8), charging U(0, 0.06), taps U(0.95, 1.05)
    on 15 % of branches); slack = bus 0; |V| at 30 % of buses, P+Q injection
    at 60 %, both-end P+Q flows on 70 % of branches, |I| at both ends of
    `current_rows` branches; telemetry = h(x_true) of the oracle (noise-free:
    the grid pins formulas, not estimates)."""
    from oracle.binding import Oracle

    rng = np.random.default_rng(seed)
    deg = np.zeros(n_bus, np.int64)
    edges = set()
    frm, to = [], []

    def add(a, b):
        frm.append(a)
        to.append(b)
        edges.add((min(a, b), max(a, b)))
        deg[a] += 1
        deg[b] += 1

    for k in range(1, n_bus):
        lo = max(0, k - 12)
        cand = [j for j in range(lo, k) if deg[j] < max_degree - 1] or [j for j in range(k) if deg[j] < max_degree]
        add(int(rng.choice(cand)), k)
    n_chords = int(0.4 * n_bus) if n_chords is None else n_chords
    tries = 0
    while n_chords > 0 and tries < 50 * n_bus:
        tries += 1
        a = int(rng.integers(0, n_bus))
        b = int(a + rng.integers(1, 10))
        if b >= n_bus or deg[a] >= max_degree or deg[b] >= max_degree or (a, b) in edges:
            continue
        add(a, b)
        n_chords -= 1
    nbr = len(frm)
    g = SimpleNamespace(n_bus=n_bus, n_branch=nbr, slack=0)
    g.bus_type = np.zeros(n_bus, np.int32)
    g.bus_type[0] = 2
    g.v_setpoint = np.ones(n_bus)
    g.br_from = np.array(frm, np.int32)
    g.br_to = np.array(to, np.int32)
    g.br_r = rng.uniform(0.01, 0.08, nbr)
    g.br_x = g.br_r * rng.uniform(3.0, 8.0, nbr)
    g.br_b = rng.uniform(0.0, 0.06, nbr)
    g.br_tap = np.ones(nbr)
    tapped = rng.choice(nbr, max(1, int(0.15 * nbr)), replace=False)
    g.br_tap[tapped] = rng.uniform(0.95, 1.05, len(tapped))
    g.br_shift = np.zeros(nbr)
    g.br_status = np.ones(nbr, np.int32)
    g.v_true = rng.uniform(0.97, 1.06, n_bus)
    g.theta_true = 0.08 * rng.standard_normal(n_bus)
    g.theta_true[0] = 0.0
    mt, ml, me = [], [], []
    for i in np.sort(rng.choice(n_bus, int(0.3 * n_bus), replace=False)):
        mt.append(0), ml.append(i), me.append(0)
    for i in np.sort(rng.choice(n_bus, int(0.6 * n_bus), replace=False)):
        mt += [2, 3]
        ml += [i, i]
        me += [0, 0]
    for k in np.sort(rng.choice(nbr, int(0.7 * nbr), replace=False)):
        mt += [4, 5, 4, 5]
        ml += [k] * 4
        me += [0, 0, 1, 1]
    for k in np.sort(rng.choice(nbr, current_rows, replace=False)):
        mt += [6, 6]
        ml += [k, k]
        me += [0, 1]
    g.m_type = np.array(mt, np.int32)
    g.m_loc = np.array(ml, np.int32)
    g.m_end = np.array(me, np.int32)
    g.n_meas = len(mt)
    g.m_sigma = np.where(g.m_type == 0, 0.004, np.where(np.isin(g.m_type, (2, 3)), 0.01, 0.008))
    o = Oracle(g)
    g.z = o.evaluate(g.v_true, g.theta_true, np.zeros(g.n_meas))["hx"]
    o.close()
    return g
