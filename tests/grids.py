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
