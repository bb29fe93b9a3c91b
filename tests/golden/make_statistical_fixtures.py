"""Writes the fixtures of the reference's statistical anchors (tests/golden/*.npz, *.json).

Reads, from a checkout of the reference (default /root/reference), the statistical CI inputs:
ci/statistical/inputs/host/argon_fcc.cif (256 Ar, P1), ci/statistical/inputs/host/RUBTAK.cif (P1,
DDEC charges), the TraPPE / UFF table ci/statistical/inputs/lennard_jones/trappe.yaml (only the
species these hosts and CO2 use), the run settings of ci/statistical/inputs/ci/{md_nvt_lj_argon,
gcmc_co2_rubtak}.yaml and the expected means and standard errors of
ci/statistical/expected/{md_nvt_lj_argon,gcmc_co2_rubtak}.yaml.  The fixtures are what the GPU
tests read (the reference checkout is not available where they run).

    python tests/golden/make_statistical_fixtures.py [reference_root]
"""

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_p1_cif(path):
    """Cell lengths / angles and the atom-site loop of a P1 CIF (labels, symbols, fractional
    coordinates and, when present, charges)."""
    cell, rows, cols, in_loop = {}, [], [], False
    for raw in open(path):
        line = raw.strip()
        if not line or line.startswith("#"):
            continue
        if line.startswith("_cell_"):
            k, v = line.split()[:2]
            cell[k] = float(v)
            continue
        if line == "loop_":
            in_loop, cols = True, []
            continue
        if in_loop and line.startswith("_"):
            cols.append(line.split()[0])
            continue
        if in_loop and cols and cols[0].startswith("_atom_site"):
            parts = line.split()
            if len(parts) == len(cols):
                rows.append(dict(zip(cols, parts)))
            continue
        in_loop = False
    lengths = [cell["_cell_length_a"], cell["_cell_length_b"], cell["_cell_length_c"]]
    angles = [cell["_cell_angle_alpha"], cell["_cell_angle_beta"], cell["_cell_angle_gamma"]]
    frac = np.array([[float(r["_atom_site_fract_x"]), float(r["_atom_site_fract_y"]), float(r["_atom_site_fract_z"])]
                     for r in rows])
    labels = [r["_atom_site_label"] for r in rows]
    charges = np.array([float(r.get("_atom_site_charge", 0.0)) for r in rows])
    return np.array(lengths), np.array(angles), frac, labels, charges


def read_lj_table(path, names):
    """sigma, epsilon of the named species from the 'parameters:' mapping (name: [sigma, eps])."""
    out, cur = {}, None
    lines = open(path).read().splitlines()
    for i, line in enumerate(lines):
        s = line.strip()
        if s.endswith(":") and line.startswith("  ") and not line.startswith("   "):
            cur = s[:-1]
            if cur in names:
                sig = float(lines[i + 1].strip().lstrip("-").strip())
                eps = float(lines[i + 2].strip().lstrip("-").strip())
                out[cur] = (sig, eps)
    return out


def read_expected(path):
    """observable -> (expected_mean, expected_sem) of an expected/*.yaml file."""
    out, cur = {}, None
    for line in open(path):
        s = line.strip()
        if line.startswith("  ") and not line.startswith("    ") and s.endswith(":"):
            cur = s[:-1]
        elif cur and s.startswith("expected_mean:"):
            out.setdefault(cur, [None, None])[0] = float(s.split(":")[1])
        elif cur and s.startswith("expected_sem:"):
            out.setdefault(cur, [None, None])[1] = float(s.split(":")[1])
    return out


def main(root):
    st = os.path.join(root, "ci", "statistical")
    # argon NVT
    lengths, angles, frac, labels, _ = read_p1_cif(os.path.join(st, "inputs", "host", "argon_fcc.cif"))
    np.savez(os.path.join(HERE, "argon_fcc.npz"), lengths=lengths, angles=angles, frac=frac)
    # RUBTAK host and the LJ rows of its species and of CO2
    lengths, angles, frac, labels, charges = read_p1_cif(os.path.join(st, "inputs", "host", "RUBTAK.cif"))
    species = sorted(set(labels))
    lj = read_lj_table(os.path.join(st, "inputs", "lennard_jones", "trappe.yaml"), set(species) | {"C_co2", "O_co2"})
    np.savez(os.path.join(HERE, "rubtak.npz"), lengths=lengths, angles=angles, frac=frac, charges=charges,
             species=np.array([species.index(x) for x in labels]), species_names=np.array(species),
             sigma=np.array([lj[x][0] for x in species]), epsilon=np.array([lj[x][1] for x in species]),
             co2_sigma=np.array([lj["C_co2"][0], lj["O_co2"][0]]),
             co2_epsilon=np.array([lj["C_co2"][1], lj["O_co2"][1]]))
    expected = {
        "md_nvt_lj_argon": {
            "source": "ci/statistical/expected/md_nvt_lj_argon.yaml; inputs ci/statistical/inputs/ci/md_nvt_lj_argon.yaml",
            "settings": {"temperature_k": 100.0, "time_step_fs": 2.0, "friction_per_fs": 1.0, "cutoff_a": 10.0,
                         "sigma_a": 3.405, "epsilon_ev": 0.01032356174398622, "tail_correction": False,
                         "warmup_steps": 5000, "steps": 5000, "integrator": "baoab_langevin"},
            "expected": read_expected(os.path.join(st, "expected", "md_nvt_lj_argon.yaml"))},
        "gcmc_co2_rubtak": {
            "source": "ci/statistical/expected/gcmc_co2_rubtak.yaml; inputs ci/statistical/inputs/ci/gcmc_co2_rubtak.yaml",
            "settings": {"pressure_pa": 10000.0, "temperature_k": 298.15, "replication": 2, "cutoff_a": 12.0,
                         "ewald_precision": 1e-6, "tail_correction": True, "warmup_cycles": 1000, "cycles": 5000,
                         "min_cycle_length": 20, "critical_temperature_k": 303.75, "critical_pressure_pa": 7840000.0,
                         "acentric_factor": 0.22394, "co2_positions": [[0, 0, 0], [-1.16, 0, 0], [1.16, 0, 0]],
                         "co2_charges": [0.7, -0.35, -0.35], "max_num_adsorbates": 100},
            "expected": read_expected(os.path.join(st, "expected", "gcmc_co2_rubtak.yaml"))},
        "tolerance_sigmas": 10.0,
        "tolerance_source": "ci/statistical/validate.py:30 (DEFAULT_TOLERANCE_SIGMAS)",
    }
    with open(os.path.join(HERE, "statistical_expected.json"), "w") as f:
        json.dump(expected, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
