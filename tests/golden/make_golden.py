"""Generate the golden fixtures in tests/golden/ from the reference checkout.

Run once where the reference is mounted (it is read-only input; nothing is executed):

    python tests/golden/make_golden.py --reference <path of the reference checkout>

The fixtures are trimmed copies of files the reference itself produced or ships:

* ``gap_transport_scan_*.csv``: rows of ``data/outputs/results/relaxtime/gap_transport_scan*.csv``
  written by ``scripts/relaxtime/run_gap_transport_scan.jl`` (p_num=12, t_num=6, iterations=40,
  MultiSeed on the first point of each (xi, muB) column, PhaseAwareContinuitySeed after it).
  Only the gap-equation columns are kept (the tau/transport columns are out of scope).
* ``dual_branch_T50.csv``: ``data/outputs/results/pnjl/dual_branch_T50.csv`` (p24/t8), both
  branches at T = 50 MeV; pins the min-Omega phase selection.
* ``tmu_scan.csv``: ``data/outputs/results/pnjl/tmu_scan.csv`` (p24/t8, 6 decimals).
* ``boundary.csv`` / ``cep.csv``: ``data/reference/pnjl/*.csv``, the phase-boundary tables the
  reference's PhaseAwareContinuitySeed reads (inputs of the seed strategy, not outputs).

Values are copied as text, digit for digit.
"""
from __future__ import annotations

import argparse
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))

GAP_COLUMNS = [
    "T_MeV", "muq_MeV", "muB_MeV", "xi", "converged", "iterations", "residual_norm",
    "Phi", "Phibar", "m_u", "m_d", "m_s", "rho_baryon", "rho_norm",
    "omega_fm4inv", "P_fm4inv", "epsilon_fm4inv", "s_fm3inv", "eps_minus_3P_over_T4",
    "n_u", "n_d", "n_s", "n_ubar", "n_dbar", "n_sbar",
]

GAP_FILES = {
    "gap_transport_scan_xi0.csv": "data/outputs/results/relaxtime/gap_transport_scan.csv",
    "gap_transport_scan_xi0p2.csv": "data/outputs/results/relaxtime/gap_transport_scan_xi0p2.csv",
    "gap_transport_scan_xim0p6to0p6.csv": "data/outputs/results/relaxtime/gap_transport_scan_xi-0p6to0p6.csv",
}

COPY_FILES = {
    "dual_branch_T50.csv": "data/outputs/results/pnjl/dual_branch_T50.csv",
    "boundary.csv": "data/reference/pnjl/boundary.csv",
    "cep.csv": "data/reference/pnjl/cep.csv",
}


def _read_scan_csv(path):
    meta, header, rows = {}, None, []
    with open(path) as fh:
        for line in fh:
            s = line.strip()
            if not s:
                continue
            if s.startswith("#"):
                body = s[1:].strip()
                if ":" in body:
                    k, v = body.split(":", 1)
                    meta[k.strip()] = v.strip()
                continue
            if header is None:
                header = s.split(",")
            else:
                rows.append(s.split(","))
    return meta, header, rows


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True)
    args = ap.parse_args()
    manifest = {}
    for out, rel in GAP_FILES.items():
        meta, header, rows = _read_scan_csv(os.path.join(args.reference, rel))
        idx = [header.index(c) for c in GAP_COLUMNS]
        with open(os.path.join(HERE, out), "w") as fh:
            fh.write(",".join(GAP_COLUMNS) + "\n")
            for r in rows:
                fh.write(",".join(r[i] for i in idx) + "\n")
        manifest[out] = {"source": rel, "rows": len(rows), "p_num": 12, "t_num": 6, "max_iter": 40,
                         "script": meta.get("script", "")}
    for out, rel in COPY_FILES.items():
        with open(os.path.join(args.reference, rel)) as fh:
            text = fh.read()
        with open(os.path.join(HERE, out), "w") as fh:
            fh.write(text)
        manifest[out] = {"source": rel}
    manifest["dual_branch_T50.csv"].update({"p_num": 24, "t_num": 8})
    # tmu_scan.csv: drop the free-text message column
    _, header, rows = _read_scan_csv(os.path.join(args.reference, "data/outputs/results/pnjl/tmu_scan.csv"))
    keep = [i for i, c in enumerate(header) if c != "message"]
    with open(os.path.join(HERE, "tmu_scan.csv"), "w") as fh:
        fh.write(",".join(header[i] for i in keep) + "\n")
        for r in rows:
            fh.write(",".join(r[i] for i in keep) + "\n")
    manifest["tmu_scan.csv"] = {"source": "data/outputs/results/pnjl/tmu_scan.csv", "rows": len(rows),
                                "p_num": 24, "t_num": 8}
    with open(os.path.join(HERE, "MANIFEST.json"), "w") as fh:
        json.dump(manifest, fh, indent=1, sort_keys=True)
        fh.write("\n")


if __name__ == "__main__":
    main()
