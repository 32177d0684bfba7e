"""Extract the reference's own known-answer data for the TCI2 path into JSON.

Reads the literal matrices of TensorCrossInterpolation.jl's tests as text
(test/test_matrixlu.jl, test/test_matrixluci.jl, and the polynomial coefficients
of test/test_integration.jl) and records, beside each, the assertion the
reference test makes about it.  Run in a checkout that has the
reference:

    python tests/golden/make_golden.py /path/to/TensorCrossInterpolation.jl

The output, tests/golden/reference_known_answers.json, is committed; the tests
never read the reference itself.
"""
import json
import os
import re
import sys


def parse_matrix_literals(text):
    """Return {line_number: matrix} for every multi-line `NAME = [ ... ]` literal."""
    lines = text.splitlines()
    out = {}
    i = 0
    while i < len(lines):
        m = re.match(r"\s*(\w+)\s*=\s*(?:([0-9.e+-]+)\s*\*\s*)?\[\s*$", lines[i])
        if m:
            scale = float(m.group(2)) if m.group(2) else 1.0
            rows = []
            j = i + 1
            while j < len(lines) and lines[j].strip() != "]":
                row = [float(x) for x in lines[j].replace(";", " ").split()]
                if row:
                    rows.append([scale * x for x in row])
                j += 1
            out[i + 1] = {"name": m.group(1), "rows": rows}
            i = j
        i += 1
    return out


def main(ref):
    lu_text = open(os.path.join(ref, "test", "test_matrixlu.jl")).read()
    luci_text = open(os.path.join(ref, "test", "test_matrixluci.jl")).read()
    lu = parse_matrix_literals(lu_text)
    luci = parse_matrix_literals(luci_text)

    def find(mats, start, name):
        for ln, m in sorted(mats.items()):
            if ln >= start and m["name"] == name:
                return m["rows"]
        raise KeyError((start, name))

    cases = [
        {"source": "test/test_matrixlu.jl:54-69", "A": find(lu, 54, "A"), "kwargs": {},
         "expect": {"left_right_approx_A": True, "L_unit_lower": True, "U_upper": True}},
        {"source": "test/test_matrixlu.jl:88-97", "A": find(lu, 88, "A"), "kwargs": {},
         "expect": {"npivot": 1}},
        {"source": "test/test_matrixlu.jl:99-121", "A": find(lu, 99, "A"), "kwargs": {"maxrank": 4},
         "expect": {"npivot": 4, "L_lower": True, "U_upper": True}},
        {"source": "test/test_matrixlu.jl:167-175", "A": [[1.0, 0.0], [0.0, 1.0]], "kwargs": {},
         "expect": {"pivoterrors": [1.0, 1.0, 0.0], "lastpivoterror": 0.0}},
        {"source": "test/test_matrixlu.jl:177-195 (maxrank=2)", "A": find(lu, 177, "A"),
         "kwargs": {"maxrank": 2}, "expect": {"n_pivoterrors": 3, "lastpivoterror_positive": True}},
        {"source": "test/test_matrixlu.jl:177-195 (abstol=0.5)", "A": find(lu, 177, "A"),
         "kwargs": {"abstol": 0.5}, "expect": {"lastpivoterror_below": 0.5}},
        {"source": "test/test_matrixlu.jl:177-195 (abstol=0)", "A": find(lu, 177, "A"),
         "kwargs": {"abstol": 0.0}, "expect": {"lastpivoterror": 0.0}},
        {"source": "test/test_matrixlu.jl:197-211", "A": find(lu, 197, "A"), "kwargs": {"abstol": 1e-3},
         "expect": {"npivot": 1, "lastpivoterror_positive": True, "max_abs_residual_below": 1e-3}},
    ]
    p = find(lu, 141, "p")
    q = find(lu, 141, "q")
    lowrank = {"source": "test/test_matrixlu.jl:141-165", "p": p, "q": q, "expect": {"npivot": 3}}
    luci_case = {"source": "test/test_matrixluci.jl:6-37", "A": find(luci, 6, "A"), "kwargs": {"maxrank": 4},
                 "expect": {"npivot": 4, "colstimespivotinv_is_leftmatrix": True}}
    tci = {
        "pivoterrors": {"source": "test/test_tensorci2.jl:27-39", "diags": [1.0, 1e-5, 0.0],
                        "localdims": [3, 3], "tolerance": 1e-8, "expect_pivoterrors": [1.0, 1e-5, 0.0]},
        "lorentz": {"source": "test/test_tensorci2.jl:247-339", "n": 5, "localdim": 10,
                    "maxbonddim2_linkdims": [2, 2, 2, 2], "globalpivot": [2, 9, 10, 5, 7],
                    "after_globalpivot_linkdims": [3, 3, 3, 3], "tol3_pivoterror_max": 2e-12,
                    "initialpivots4": [[1, 1, 1, 1, 1], [10, 8, 10, 4, 4], [5, 4, 8, 9, 3], [7, 7, 10, 5, 9],
                                       [7, 7, 10, 5, 9]]},
        "convergencecriterion": {
            "source": "test/test_tensorci2.jl:504-554",
            "cases": [
                {"ranks": [1, 2], "errors": [1e-2, 1e-5], "ngp": [0, 0], "tol": 1e-4, "maxbonddim": 4,
                 "ncheck": 3, "expect": False},
                {"ranks": [1, 2, 2, 2], "errors": [1e-2, 1e-5, 1e-5, 1e-5], "ngp": [0, 0, 0, 0], "tol": 1e-4,
                 "maxbonddim": 4, "ncheck": 3, "expect": True},
                {"ranks": [1, 2, 2, 2], "errors": [1e-2, 1e-2, 1e-5, 1e-5], "ngp": [0, 0, 0, 0], "tol": 1e-4,
                 "maxbonddim": 4, "ncheck": 3, "expect": False},
                {"ranks": [1, 2, 2, 2], "errors": [1e-2, 1e-2, 1e-2, 1e-2], "ngp": [0, 0, 0, 0], "tol": 1e-4,
                 "maxbonddim": 2, "ncheck": 3, "expect": True},
                {"ranks": [1, 2, 2, 2], "errors": [1e-2, 1e-2, 1e-2, 1e-2], "ngp": [0, 1, 1, 1], "tol": 1e-4,
                 "maxbonddim": 2, "ncheck": 3, "expect": True},
            ]},
    }
    integ_text = open(os.path.join(ref, "test", "test_integration.jl")).read()
    m = re.search(r"coefficients\s*=\s*\[(.*?)\]", integ_text, re.S)
    coeffs = [float(x) for x in m.group(1).replace("\n", " ").split(",") if x.strip()]
    m10 = re.search(r"Iref\s*=\s*([-0-9.e]+)", integ_text)
    integration = {"source": "test/test_integration.jl:6-28", "coefficients": coeffs, "N": 5,
                   "expect": "integrate(f, a, b) ≈ prod(P(b) - P(a)) for f(x) = prod(p.(x)), P' = p; "
                             "[0,1]^5 and a random box",
                   "tenD": {"source": "test/test_integration.jl:61-70",
                            "f": "1000 cos(10 sum(x.^2)) exp(-sum(x)^4 / 1000)", "N": 10, "a": -1.0, "b": 1.0,
                            "GKorder": 15, "tolerance": 1e-8, "Iref": float(m10.group(1)), "abs_tol": 1e-3}}
    util = {"optfirstpivot": {"source": "test/test_util.jl:29-37",
                              "f": "2^2 (v3 - 1) + 2^1 (v2 - 1) + 2^0 (v1 - 1)", "localdims": [2, 2, 2],
                              "firstpivot": [1, 1, 1], "expect": [2, 2, 2]}}
    contraction = {"source": "test/test_contraction.jl:30-47, 68-99, 148-183",
                   "mpo_mpo": {"bonddims_a": [1, 2, 3, 2, 1], "bonddims_b": [1, 2, 3, 2, 1],
                               "localdims1": [2, 2, 2, 2], "localdims2": [3, 3, 3, 3], "localdims3": [2, 2, 2, 2]},
                   "f": [None, "2x"], "algorithms": ["TCI", "naive"],
                   "expect": "_tomat(contract(a, b)) ≈ _tomat(a) * _tomat(b) (≈ f.(...) with f)"}
    out = {"reference": "TensorCrossInterpolation.jl 0.9.19", "rrlu": cases, "rrlu_lowrank": lowrank,
           "luci": luci_case, "tci2": tci, "integration": integration, "util": util,
           "contraction": contraction}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_known_answers.json")
    with open(dst, "w") as fh:
        json.dump(out, fh, indent=1)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/TensorCrossInterpolation.jl")
    main(sys.argv[1])
