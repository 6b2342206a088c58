"""Builds the golden fixtures in this folder from the mumfim source tree.

Run once where the reference tree is present:

    python tests/golden/make_golden.py /path/to/mumfim

It reads the reference's own test data and known answers and writes them as
JSON, so the tests run without the reference tree:

* network_2_7.json -- test/microscale/fiber_networks/Network_2_7.txt(.params),
  the deformation gradient and damping of test/microscale/fiber_only.yaml, and
  the stress and FD stiffness the reference printed for that case in
  test/microscale/before-refactor-outputs/{explicit_cpu,explicit_gpu,implicit}_out.txt.
* reorder_kat.json -- the boundary-last permutation known answer of
  test/microscale/test_reorder_mesh.cc:9-67.
"""
from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from mumfim_gb300.network_io import load_network  # noqa: E402


def _floats(line: str) -> list[float]:
    return [float(t) for t in line.split()]


def parse_run_output(path: str) -> dict:
    """Stress blocks ('Stress from run' + 3 rows) and the 6x6 stiffness that
    follows each, plus the 'Took:' wall time."""
    with open(path) as fh:
        lines = [l.rstrip("\n") for l in fh]
    stresses, stiffnesses = [], []
    took = None
    i = 0
    while i < len(lines):
        if lines[i].startswith("Stress from run"):
            rows = [_floats(lines[i + k]) for k in (1, 2, 3)]
            stresses.append(rows)
            # the stiffness block: the next 6 lines of 6 numbers after a blank
            j = i + 4
            while j < len(lines) and not lines[j].strip():
                j += 1
            block = []
            while j < len(lines) and len(block) < 6:
                vals = _floats(lines[j]) if re.match(r"^\s*[-0-9.]", lines[j]) else []
                if len(vals) == 6:
                    block.append(vals)
                    j += 1
                else:
                    break
            if len(block) == 6:
                stiffnesses.append(block)
            i = j
            continue
        m = re.match(r"Took:\s*([0-9.eE+-]+)", lines[i])
        if m:
            took = float(m.group(1))
        i += 1
    return {"stress": stresses, "stiffness": stiffnesses, "took_s": took}


def parse_yaml_F(path: str) -> list[float]:
    with open(path) as fh:
        for line in fh:
            s = line.strip()
            if s.startswith("Deformation Gradient:"):
                inner = s.split("[", 1)[1].split("]", 1)[0]
                return [float(t) for t in inner.split(",")]
    raise RuntimeError("no deformation gradient in " + path)


def parse_yaml_scalar(path: str, key: str) -> float:
    with open(path) as fh:
        for line in fh:
            s = line.strip()
            if s.startswith(key + ":"):
                return float(s.split(":", 1)[1].split("#")[0])
    raise RuntimeError(f"no {key} in {path}")


def parse_reorder_kat(path: str) -> dict:
    with open(path) as fh:
        src = fh.read()

    def arr(name: str) -> list[float]:
        m = re.search(r"std::array<[^>]*>\s*" + name + r"\s*(?:=\s*)?\{([^}]*)\}", src)
        if not m:
            raise RuntimeError("array " + name + " not found")
        return [float(t) for t in m.group(1).replace("\n", " ").split(",") if t.strip()]

    nverts = int(re.search(r"int\s+nverts\s*=\s*(\d+)", src).group(1))
    return {
        "source": "test/microscale/test_reorder_mesh.cc:9-67",
        "n_verts": nverts,
        "fixed_verts": [int(v) for v in arr("fixed_verts")],
        "initial_connectivity": [int(v) for v in arr("initial_connectivity")],
        "final_connectivity": [int(v) for v in arr("final_connectivity")],
        # coordinates(row, col) = 3*row + col before the permutation
        "final_coordinates": arr("final_coordinates"),
    }


def main(ref: str) -> None:
    micro = os.path.join(ref, "test", "microscale")
    net_path = os.path.join(micro, "fiber_networks", "Network_2_7.txt")
    net = load_network(net_path)
    yaml_path = os.path.join(micro, "fiber_only.yaml")
    outs = {}
    for name in ("explicit_cpu_out", "explicit_gpu_out", "implicit_out"):
        outs[name] = parse_run_output(os.path.join(micro, "before-refactor-outputs", name + ".txt"))
    r0 = net.reactions[0]
    golden = {
        "source": {
            "network": "test/microscale/fiber_networks/Network_2_7.txt(.params)",
            "case": "test/microscale/fiber_only.yaml",
            "outputs": "test/microscale/before-refactor-outputs/*_out.txt",
        },
        "coords": net.coords.tolist(),
        "connectivity": net.connectivity.tolist(),
        "reaction": {"law": r0.law, "radius": r0.radius, "youngs_modulus": r0.youngs_modulus,
                     "density": r0.density, "B": r0.B, "length_ratio_trns": r0.length_ratio_trns},
        "F": parse_yaml_F(yaml_path),
        "visc_damp_coeff": parse_yaml_scalar(yaml_path, "Viscous Damping Factor"),
        "crit_time_scale_factor": parse_yaml_scalar(yaml_path, "Critical Time Scale Factor"),
        "outputs": outs,
    }
    with open(os.path.join(HERE, "network_2_7.json"), "w") as fh:
        json.dump(golden, fh)
    with open(os.path.join(HERE, "reorder_kat.json"), "w") as fh:
        json.dump(parse_reorder_kat(os.path.join(micro, "test_reorder_mesh.cc")), fh, indent=1)
    print("wrote network_2_7.json, reorder_kat.json")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: python make_golden.py <path of the mumfim source tree>")
    main(sys.argv[1])
