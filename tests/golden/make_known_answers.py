"""Known-answer fixtures from the reference's own tests.

Run where the reference tree is available (it reads /root/reference):

    python tests/golden/make_known_answers.py

The reference's test_calc/test_properties_MgO.py evaluates two shipped
potentials (tests/test_calc/files/mlps/polymlp.yaml.pair.MgO and
polymlp.yaml.gtinv.MgO) on the displaced rocksalt cell
tests/test_calc/files/poscars/POSCAR.RS.MgO and asserts energy, forces and
stresses (GPa) at fixed values (test_eval1, test_eval2).  This script copies
those three data files into tests/golden/known_answers/, takes the asserted
values from the test source (the literal assignments energy_true, forces_true,
stresses_true of each test function, read with `ast`, not executed) into
known_answers.json, and writes the invariant tables the gtinv potential needs
(order 3, l_max (4, 4)) with the reference's Readgtinv (oracle/_ref).
"""

import ast
import json
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

REF_TESTS = "/root/reference/tests/test_calc"
OUT = os.path.join(HERE, "known_answers")
FILES = {
    "polymlp.yaml.pair.MgO": "files/mlps/polymlp.yaml.pair.MgO",
    "polymlp.yaml.gtinv.MgO": "files/mlps/polymlp.yaml.gtinv.MgO",
    "POSCAR.RS.MgO": "files/poscars/POSCAR.RS.MgO",
}
# reference test function -> (potential, structure)
CASES = {"test_eval1": ("polymlp.yaml.pair.MgO", "POSCAR.RS.MgO"),
         "test_eval2": ("polymlp.yaml.gtinv.MgO", "POSCAR.RS.MgO")}


def asserted_values(path):
    tree = ast.parse(open(path).read())
    out = {}
    for fn in tree.body:
        if not isinstance(fn, ast.FunctionDef) or fn.name not in CASES:
            continue
        vals = {}
        for node in ast.walk(fn):
            if isinstance(node, ast.Assign) and len(node.targets) == 1 and isinstance(node.targets[0], ast.Name):
                name = node.targets[0].id
                if name in ("energy_true", "forces_true", "stresses_true"):
                    vals[name] = ast.literal_eval(node.value)
        pot, poscar = CASES[fn.name]
        out[fn.name] = {"potential": pot, "structure": poscar, "energy": vals["energy_true"],
                        "forces": vals["forces_true"], "stresses_gpa": vals["stresses_true"],
                        "tolerances": {"energy_rel": 1e-8, "forces_abs": 1e-6, "stresses_gpa_abs": 1e-5}}
    return out


def main():
    os.makedirs(OUT, exist_ok=True)
    for name, rel in FILES.items():
        shutil.copyfile(os.path.join(REF_TESTS, rel), os.path.join(OUT, name))
        print("copied", name)
    answers = asserted_values(os.path.join(REF_TESTS, "test_properties_MgO.py"))
    with open(os.path.join(OUT, "known_answers.json"), "w") as f:
        json.dump({"source": "tests/test_calc/test_properties_MgO.py", "cases": answers}, f, indent=1)
    print("wrote known_answers.json:", sorted(answers))

    from oracle import ref
    from pypolymlp_gb300.params import gtinv_file

    order, maxl = 3, (4, 4)
    l_comb, lm_seq, lm_coeffs = ref.readgtinv(order, maxl)
    with open(gtinv_file(order, maxl), "w") as f:
        json.dump({"order": order, "maxl": list(maxl), "version": 1, "l_comb": l_comb, "lm_seq": lm_seq,
                   "lm_coeffs": lm_coeffs}, f, separators=(",", ":"))
    print("wrote", gtinv_file(order, maxl))


if __name__ == "__main__":
    main()
