"""Writes reference_known_answers.json: the numbers the reference itself asserts or prints
for the DMRG path, taken verbatim from its test file and its example notebook (Julia is not
available here, so the reference cannot be run; these are its own recorded answers).

    python tests/golden/extract_known_answers.py /root/reference

* test/unit/dmrg.jl — the four `energy / n ≈ value atol = tol` assertions (Ising n=10, h=J=1,
  10 sweeps) with the start state and method of their testset.
* examples/dmrg.ipynb — the printed per-call energy vectors of its two runs (Ising n=100,
  h=J=1, χ=128: Dmrg1 from rand(MPS), Dmrg2 from the product state |0…0⟩).
"""

import json
import os
import re
import sys


def dmrg_tests(root):
    path = "test/unit/dmrg.jl"
    src = open(os.path.join(root, path)).read().split("\n")
    out, start, method, maxdim = [], None, None, None
    for ln, line in enumerate(src, 1):
        if "ProductState(fill([1, 0], n))" in line:
            start = "product"
        elif "delta[1, 1, 1] = 1.0" in line:
            start = "delta"
        m = re.search(r"method=Tenet\.DMRG\.(Dmrg[12])\(\)(?:, maxdim=(\d+))?", line)
        if m:
            method, maxdim = m.group(1), int(m.group(2)) if m.group(2) else None
        m = re.search(r"energy / n ≈ (-?[0-9.]+) atol = ([0-9.e-]+)", line)
        if m:
            out.append({"source": f"{path}:{ln}", "start": start, "method": method, "maxdim": maxdim,
                        "energy_per_site": float(m.group(1)), "atol": float(m.group(2))})
    return out


def notebook(root):
    path = "examples/dmrg.ipynb"
    nb = json.load(open(os.path.join(root, path)))
    runs = {}
    for k, cell in enumerate(nb["cells"]):
        if cell["cell_type"] != "code":
            continue
        code = "".join(cell["source"])
        for o in cell.get("outputs", []):
            txt = "".join(o.get("text", [])) or "".join(o.get("data", {}).get("text/plain", []))
            if "Vector{Float64}" not in txt:
                continue
            vals = [float(v) for v in re.findall(r"-?\d+\.\d+", txt.split(":", 1)[1])]
            name = "dmrg1_rand" if "Dmrg1" in code else "dmrg2_product"
            runs[name] = {"source": f"{path} cell {k}", "energies_per_call": vals}
    return runs


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    data = {"dmrg_tests": dmrg_tests(root), "dmrg_notebook": notebook(root),
            "notebook_workload": {"n": 100, "h": 1.0, "J": 1.0, "maxdim": 128, "calls": 10,
                                  "call": "dmrg!(psi, H, 1; method, maxdim = 128)"}}
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "reference_known_answers.json"), "w") as f:
        json.dump(data, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
