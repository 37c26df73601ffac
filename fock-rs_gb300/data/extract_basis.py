"""Extract the basis-set data the hot path needs into one compact JSON file.

The reference ships Basis Set Exchange (BSE) JSON files under
``basis_set/src/data/*.json`` and expands them in ``basis_set/src/lib.rs:79-118``.
Only H, C, N and O of STO-3G, 6-31G and 6-31G* are needed by the benchmark
molecules, so this script copies those shells (exponents and contraction
coefficients as the original decimal strings, so parsing is bit-identical)
into ``basis_sets.json`` beside it.  It reads the reference checkout given as
the first argument and is run once, by hand; the output is committed.
"""
import json
import os
import sys

SETS = {"STO-3G": "STO-3G.json", "6-31G": "6-31G.json", "6-31G*": "6-31G_st.json"}
ELEMENTS = ["1", "6", "7", "8"]


def main(ref_root):
    out = {}
    for name, fname in SETS.items():
        src = json.load(open(os.path.join(ref_root, "basis_set/src/data", fname)))
        out[name] = {}
        for el in ELEMENTS:
            shells = []
            for s in src["elements"][el]["electron_shells"]:
                shells.append({
                    "angular_momentum": s["angular_momentum"],
                    "function_type": s["function_type"],
                    "exponents": s["exponents"],
                    "coefficients": s["coefficients"],
                })
            out[name][el] = shells
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "basis_sets.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", dst)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
