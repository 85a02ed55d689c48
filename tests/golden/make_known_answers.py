"""Writes reference_known_answers.json: the known-answer cases of the
reference's own unit tests for the DC-PSE building blocks, transcribed from
their source (paths relative to the openfpm_numerics tree).

Run from the repository root:  python tests/golden/make_known_answers.py
"""
import json
import os

CASES = {
    # src/DCPSE/tests/MonomialBasis_unit_tests.cpp:13-53
    "monomial_order": [
        {"exps": [1, 2, 3], "order": 6},
        {"exps": [0, 0, 0], "order": 0},
        {"exps": [5, 5, 5], "order": 15},
    ],
    # MonomialBasis_unit_tests.cpp:55-71
    "monomial_evaluate": [
        {"exps": [1, 1, 1], "x": [5, 3, 2], "value": 30.0},
        {"exps": [5, 3, 2], "x": [2, 2, 2], "value": 1024.0},
    ],
    # MonomialBasis_unit_tests.cpp:73-113
    "monomial_derivative": [
        {"exps": [6, 6, 6], "d": [3, 0, 0], "out_exps": [3, 6, 6], "out_scalar": 120},
        {"exps": [6, 6, 6], "d": [0, 3, 0], "out_exps": [6, 3, 6], "out_scalar": 120},
        {"exps": [6, 6, 6], "d": [0, 0, 3], "out_exps": [6, 6, 3], "out_scalar": 120},
        {"exps": [6, 6, 6], "d": [7, 0, 0], "out_exps": [0, 6, 6], "out_scalar": 0},
        {"exps": [6, 6, 6], "d": [0, 7, 0], "out_exps": [6, 0, 6], "out_scalar": 0},
        {"exps": [6, 6, 6], "d": [0, 0, 7], "out_exps": [6, 6, 0], "out_scalar": 0},
    ],
    # MonomialBasis_unit_tests.cpp:115-168 (membership; :139-168 also pins the size)
    "basis_2d": [
        {"sig": [1, 0], "order": 2, "contains": [[0, 0], [1, 0], [0, 1], [1, 1], [2, 0], [0, 2]], "size": None},
        {"sig": [1, 1], "order": 2,
         "contains": [[1, 0], [0, 1], [1, 1], [2, 0], [0, 2], [2, 1], [1, 2], [3, 0], [0, 3]], "size": 9},
    ],
    # src/DCPSE/tests/Vandermonde_unit_tests.cpp:19-72 (basis of sig (1,0), r=2)
    "row_builder": [
        {"x": [2, 2], "eps": 2, "pattern": "all_ones"},
        {"x": [1, 0], "eps": 1, "pattern": "one_where_no_y"},
        {"x": [0, 1], "eps": 1, "pattern": "one_where_no_x"},
    ],
    # src/DCPSE/tests/DcpseRhs_unit_tests.cpp:16-109: b_i = sign * (D^sig m_i)(0)
    "rhs": [
        {"sig": [1, 0], "order": 2, "sign": -1, "size": 6},
        {"sig": [1, 1], "order": 2, "sign": 1, "size": 9},
        {"sig": [2, 2], "order": 2, "sign": 1, "size": 20},
    ],
    # basis sizes used by the benchmark configurations (3D Gradient / Laplacian)
    "basis_sizes": [
        {"dim": 2, "sig": [2, 0], "order": 2, "size": 9},
        {"dim": 3, "sig": [1, 0, 0], "order": 2, "size": 10},
        {"dim": 3, "sig": [2, 0, 0], "order": 2, "size": 19},
    ],
    # analytic error bars of the reference's DC-PSE tests
    "analytic": [
        {"name": "Dcpse_2D_test", "src": "src/DCPSE/tests/Dcpse_unit_tests.cpp:36-133",
         "nside": 40, "rcut_h": 3.1, "sig": [1, 0], "field": "sin(x)", "tol": "2*(2h)^2"},
        {"name": "Dcpse_3D_test", "src": "src/DCPSE/tests/Dcpse_unit_tests.cpp:243-337",
         "nside": 40, "rcut_h": 3.1, "sig": [0, 0, 1], "field": "sin(z)", "tol": "(3h)^2"},
        {"name": "dcpse_op_tests", "src": "src/DCPSE/DCPSE_op/tests/DCPSE_op_test_base_tests.cpp:30-101",
         "nside": 80, "box": "2pi", "rcut_h": 3.9, "expr": "2Dx+Dy of sin(x)+sin(y)", "worst": 0.03},
        {"name": "dcpse_op_test_lap", "src": "src/DCPSE/DCPSE_op/tests/DCPSE_op_test_base_tests.cpp:394-467",
         "nside": 163, "box": "2pi", "rcut_h": 3.9, "expr": "Lap of sin(x)+sin(y)", "worst": 0.3},
    ],
}

if __name__ == "__main__":
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_known_answers.json")
    with open(out, "w") as fh:
        json.dump(CASES, fh, indent=1)
    print(out)
