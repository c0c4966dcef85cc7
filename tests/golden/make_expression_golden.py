"""Writes the boundary-condition expression fixture from the reference's OWN expression evaluator.

`make -C oracle ref` compiles cpp/expression.cpp (Expression::init and ::evaluate) into oracle/_ref/libref_kdtree.so.
This script evaluates a list of expressions with it, at three (x, y, t) points, the way the reference's
VelocityDirichlet::eval / PressureDirichlet::eval call it (cpp/grid.cpp:80-94: float variables), and stores the
float results and, for texts the reference rejects without ending the process, which step rejects them ("init" or
"evaluate").  The restatement in oracle/ and the product's evaluator are checked against it where the reference
checkout does not exist.

Two malformed texts are left out on purpose: "(1+2" stops the reference process in an assert
(getNumOperatorArgs, cpp/expression.cpp:123) and "1+*" does not terminate in Expression::init.

    NSFEM_REFERENCE_DIR=<reference checkout> python tests/golden/make_expression_golden.py
"""
from __future__ import annotations

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

OUT = os.path.join(HERE, "ref_expressions.json")

EXPRESSIONS = [
    "4*1.5*y*(0.41-y)/(0.41*0.41)", "-2^2", "2^-1", "2^3^2", "sin(Pi/2)+cos(0)*E", "1-x-y*3/2", "-(x+1)*-2",
    "4*y*(1-y)", "0", "1e-3*x", "4*1.5*y*(0.41-y)/(0.41*0.41)*sin(Pi*t/8)", "-x^2^-1+t", "2^-t*cos(x-y*t)/3",
    "1-t/2*-x", "E^(t*x)-Pi*-(y)", "(x+y)*(x-y)^2/(1+t)", "sin(cos(t))*-3^2", "0.15*t-x/y/t", "((x))", "x*-y^2",
    "-sin(-x)*cos(y)^2", "1.5e2/x-2.5E-1*y", "3-2-1", "16/4/2", "2*3^2", "-(-(-x))",
]
REJECTED = ["z+1", "sin 3", "x$"]
POINTS = [(0.3, 0.2, 0.05), (1.0, 0.37, 2.5), (0.7, 0.1, 1e-3)]


def main():
    if not os.environ.get("NSFEM_REFERENCE_DIR"):
        raise SystemExit("set NSFEM_REFERENCE_DIR to the reference checkout")
    oracle.build(ref=True)
    values = {e: [oracle.ref_evaluate_expression(e, *p) for p in POINTS] for e in EXPRESSIONS}
    rejected = {}
    for e in REJECTED:
        try:
            oracle.ref_evaluate_expression(e, *POINTS[0])
        except ValueError as err:
            rejected[e] = "init" if "(init)" in str(err) else "evaluate"
        else:
            raise SystemExit(f"the reference accepts {e!r}")
    with open(OUT, "w") as f:
        json.dump({"points": POINTS, "values": values, "rejected": rejected}, f, indent=1)
    print(len(values), "expressions,", len(rejected), "rejected")


if __name__ == "__main__":
    main()
