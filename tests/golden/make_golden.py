"""Extract the reference's shipped run outputs into small test fixtures.

Run once in a checkout that has the reference next to it:

    python tests/golden/make_golden.py /path/to/ProjecTracer

Inputs (all produced by the reference's own run of its shipped inputs.nml with 2 OpenMP threads):
stdout (known-answer values), stats.dat (basics.f90:427-428 format), T10000 (t=0 snapshot,
main.f90:396-397 format), P10000 (lateral averages, main.f90:414-422) and inputs.nml.
Outputs: reference_run.json, T10000_subset.npz and snapshot_t0_lines.json in this directory.
"""

from __future__ import annotations

import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from projectracer_gb300.namelist import read_namelist  # noqa: E402

STATS_COLS = ["time", "Tavg", "vrms", "Nu", "Nu_bot", "RaT_avg", "mobility", "strain_max", "q1", "q2",
              "q3", "q4", "empty_cells", "tracer_min", "tracer_max", "Cavg", "entrainment"]


def main(ref: str) -> None:
    out: dict = {}
    rows = []
    with open(os.path.join(ref, "stats.dat")) as fh:
        for line in fh:
            vals = line.split()
            if len(vals) == len(STATS_COLS):
                rows.append({k: (int(v) if k in ("empty_cells", "tracer_min", "tracer_max") else float(v))
                             for k, v in zip(STATS_COLS, vals)})
    out["stats"] = rows
    kat = {}
    with open(os.path.join(ref, "stdout")) as fh:
        text = fh.read()
    kat["RKC1_stability"] = float(re.search(r"RKC1_stability=\s*(\S+)", text).group(1))
    m = re.search(r"Tbot_iso,Ttop_iso=\s*(\S+)\s+(\S+)", text)
    kat["Tbot_iso"], kat["Ttop_iso"] = float(m.group(1)), float(m.group(2))
    m = re.search(r"subD,supD,ngrid=\s*(\d+)\s+(\d+)\s+(\d+)", text)
    kat["subD"], kat["supD"], kat["ngrid"] = int(m.group(1)), int(m.group(2)), int(m.group(3))
    kat["ntr"] = int(re.search(r"ntr=\s*(\d+)", text).group(1))
    kat["Nthreads"] = int(re.search(r"Nthreads=\s*(\d+)", text).group(1))
    m = re.search(r"Entrainment Calculation:\s*(\d+)\s+(\S+)", text)
    kat["kent"], kat["zent"] = int(m.group(1)), float(m.group(2))
    kat["T_smoothing"] = float(re.search(r"T Smoothing Parameter:\s*(\S+)", text).group(1))
    kat["C_smoothing"] = float(re.search(r"C Smoothing Parameters:\s*(\S+)", text).group(1))
    out["stdout"] = kat
    out["namelist"] = read_namelist(os.path.join(ref, "inputs.nml"))
    # lateral averages: z, Tlat (columns 1-2 of P10000)
    prof = []
    with open(os.path.join(ref, "P10000")) as fh:
        for line in fh:
            v = line.split()
            if len(v) == 4:
                prof.append([float(v[0]), float(v[1])])
    out["P10000_z_Tlat"] = prof
    with open(os.path.join(HERE, "reference_run.json"), "w") as fh:
        json.dump(out, fh, indent=1)
    # T10000: x, z, T, SF, u, w, stress, vis, Tvis, nempty, Cnew, Cvis (i outer, k inner)
    data = []
    with open(os.path.join(ref, "T10000")) as fh:
        for line in fh:
            v = line.split()
            if len(v) >= 12:
                data.append([float(x) for x in v[:12]])
    A = np.array(data)
    n = int(round(np.sqrt(A.shape[0])))
    i = np.repeat(np.arange(n), n)
    k = np.tile(np.arange(n), n)
    keep = ((i % 5) == 0) & ((k % 5) == 0) | (k == 1) | (k == n - 2)
    np.savez_compressed(os.path.join(HERE, "T10000_subset.npz"), i=i[keep], k=k[keep], cols=A[keep])
    # the snapshot files as printed (every 37th line of T10000 with its line number, all of P10000),
    # for the snapshot writer's edit descriptors
    with open(os.path.join(ref, "T10000")) as fh:
        tl = fh.read().split("\n")
    with open(os.path.join(ref, "P10000")) as fh:
        pl = fh.read().split("\n")
    sample = {"T10000": [[n, tl[n]] for n in range(0, len(tl), 37) if tl[n]], "P10000": [ln for ln in pl if ln]}
    with open(os.path.join(HERE, "snapshot_t0_lines.json"), "w") as fh:
        json.dump(sample, fh, indent=0)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the reference checkout>")
    main(sys.argv[1])
