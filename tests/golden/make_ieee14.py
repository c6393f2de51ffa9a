"""Extract the SLE Engine's IEEE 14-bus fixture into this repository.

Reads the reference's ``data/ieee14bus.h`` (the only fixture the reference
ships: model at :68-270, "true" telemetry at :284-330) and writes

  tests/golden/ieee14.json
      buses / branches / measurements in insertion order plus the true
      telemetry keyed by measurement id;
  state_estimation_with_cuda_gb300/csrc/api/ieee14_data.inc
      the same model as a C table, compiled into sle_LoadIEEE14Bus.

Usage:  python tests/golden/make_ieee14.py path/to/reference
The reference checkout is only needed to regenerate; both outputs are
committed.
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))

BUS_TYPES = {"PQ": 0, "PV": 1, "SLACK": 2}
MEAS_TYPES = {"V_MAG": 0, "V_ANGLE": 1, "P_INJECTION": 2, "Q_INJECTION": 3, "P_FLOW": 4,
              "Q_FLOW": 5, "I_MAG": 6, "P_PSEUDO": 7, "Q_PSEUDO": 8}


def num(tok):
    return float(tok.strip().rstrip("f"))


def parse(src):
    buses, branches, meas = [], [], []
    for m in re.finditer(r'BusDescriptor\(\s*"([^"]+)",\s*([-\d.]+f?),\s*BusType::(\w+),\s*([-\d.]+f?),'
                         r'\s*([-\d.]+f?),\s*([-\d.]+f?)\)', src):
        buses.append({"id": m.group(1), "base_kv": num(m.group(2)), "type": BUS_TYPES[m.group(3)],
                      "v_setpoint": num(m.group(4)), "p": num(m.group(5)), "q": num(m.group(6))})
    for m in re.finditer(r'BranchDescriptor\(\s*"([^"]+)",\s*"([^"]+)",\s*"([^"]+)",\s*([-\d.]+f?),\s*([-\d.]+f?),'
                         r'\s*([-\d.]+f?),\s*([-\d.]+f?),\s*([-\d.]+f?),\s*([-\d.]+f?),\s*(true|false)\)', src):
        branches.append({"id": m.group(1), "from": m.group(2), "to": m.group(3), "r": num(m.group(4)),
                         "x": num(m.group(5)), "b": num(m.group(6)), "g": num(m.group(7)),
                         "tap": num(m.group(8)), "shift": num(m.group(9)), "xfmr": m.group(10) == "true"})
    # |V| at every bus from the loop (ieee14bus.h:197-204)
    loop = re.search(r'for \(int i = 1; i <= (\d+); \+\+i\).*?MeasurementType::V_MAG.*?BranchEnd::FROM,\s*([-\d.]+f?)',
                     src, re.S)
    for i in range(1, int(loop.group(1)) + 1):
        meas.append({"id": "V%d" % i, "type": 0, "location": "Bus%d" % i, "end": 0, "sigma": num(loop.group(2)),
                     "pseudo": False})
    for m in re.finditer(r'MeasurementDescriptor\(\s*"([^"]+)",\s*MeasurementType::(\w+),\s*"([^"]+)",'
                         r'\s*BranchEnd::(\w+),\s*([-\d.]+f?),\s*([-\d.]+f?),\s*([-\d.]+f?),\s*(true|false)\)', src):
        meas.append({"id": m.group(1), "type": MEAS_TYPES[m.group(2)], "location": m.group(3),
                     "end": 0 if m.group(4) == "FROM" else 1, "sigma": num(m.group(5)),
                     "pseudo": m.group(8) == "true"})
    # true telemetry (ieee14bus.h:284-330)
    arrays = {}
    for m in re.finditer(r'(voltages|p_inj|q_inj|p_flow|q_flow)\[(\d+)\]\s*=\s*([-\d.]+)f;', src):
        arrays.setdefault(m.group(1), {})[int(m.group(2))] = float(m.group(3))
    true = {}
    for i, v in sorted(arrays["voltages"].items()):
        true["V%d" % (i + 1)] = v
    inj_p_ids = [x["id"] for x in meas if x["type"] == 2]
    inj_q_ids = [x["id"] for x in meas if x["type"] == 3]
    pf_ids = [x["id"] for x in meas if x["type"] == 4]
    qf_ids = [x["id"] for x in meas if x["type"] == 5]
    for ids, key in ((inj_p_ids, "p_inj"), (inj_q_ids, "q_inj"), (pf_ids, "p_flow"), (qf_ids, "q_flow")):
        for i, v in sorted(arrays[key].items()):
            true[ids[i]] = v
    for x in meas:  # zero-injection pseudo measurements carry 0
        if x["pseudo"]:
            true[x["id"]] = 0.0
    return {"buses": buses, "branches": branches, "measurements": meas, "true_telemetry": true}


def c_table(d):
    out = ["/* Generated by tests/golden/make_ieee14.py from the SLE Engine IEEE 14-bus fixture. */"]
    out.append("static const Ieee14Bus kIeee14Buses[] = {")
    for b in d["buses"]:
        out.append('    {"%s", %r, %d, %r, %r, %r},' % (b["id"], b["base_kv"], b["type"], b["v_setpoint"], b["p"], b["q"]))
    out.append("};")
    out.append("static const Ieee14Branch kIeee14Branches[] = {")
    for b in d["branches"]:
        out.append('    {"%s", "%s", "%s", %r, %r, %r, %r, %r, %r, %d},' % (
            b["id"], b["from"], b["to"], b["r"], b["x"], b["b"], b["g"], b["tap"], b["shift"], int(b["xfmr"])))
    out.append("};")
    out.append("static const Ieee14Meas kIeee14Meas[] = {")
    for m in d["measurements"]:
        out.append('    {"%s", %d, "%s", %d, %r, %d},' % (m["id"], m["type"], m["location"], m["end"], m["sigma"],
                                                         int(m["pseudo"])))
    out.append("};")
    return "\n".join(out) + "\n"


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_ieee14.py path/to/reference")
    ref = sys.argv[1]
    with open(os.path.join(ref, "data", "ieee14bus.h")) as fh:
        src = fh.read()
    d = parse(src)
    assert len(d["buses"]) == 14 and len(d["branches"]) == 20, (len(d["buses"]), len(d["branches"]))
    with open(os.path.join(HERE, "ieee14.json"), "w") as fh:
        json.dump(d, fh, indent=1)
    inc = os.path.join(REPO, "state_estimation_with_cuda_gb300", "csrc", "api", "ieee14_data.inc")
    with open(inc, "w") as fh:
        fh.write(c_table(d))
    print("buses %d branches %d measurements %d telemetry %d" % (
        len(d["buses"]), len(d["branches"]), len(d["measurements"]), len(d["true_telemetry"])))


if __name__ == "__main__":
    main()
