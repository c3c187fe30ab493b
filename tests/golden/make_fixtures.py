"""Generate the committed golden fixtures under tests/golden/.

Run in the build container, where the reference checkout is readable:

    python tests/golden/make_fixtures.py /path/to/reference

* ``reference_testvals.json``: the ``testval``/golden numbers of the reference
  examples and tests used to pin the oracle, read from the reference sources as
  text, each with its file:line.
* ``bernoulli_kat.npz``: the known-answer vectors of
  ``test/test010_bernoulli.jl``: B(x) = x/(exp(x)-1) on (a stride of) the ranges
  -1:1.00001e-5:1 and -100:1.00001e-3:100, evaluated in 60-digit decimal
  arithmetic (the reference evaluates them in BigFloat).
"""
import decimal
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = None  # the reference checkout, the required command-line argument

EXAMPLES = {
    # the value is inline in runtests: @test main() ≈ value
    "Example101_Laplace1D": r"main\(\)\s*≈\s*([-0-9.e]+)",
    "Example102_StationaryConvectionDiffusion1D": r"testval\s*=\s*([-0-9.e]+)",
    "Example105_NonlinearPoisson1D": r"testval\s*=\s*([-0-9.e]+)",
    "Example107_NonlinearStorage1D": r"testval\s*=\s*([-0-9.e]+)",
    "Example106_NonlinearDiffusion1D": r"testval\s*=\s*([-0-9.e]+)",
    "Example110_ReactionDiffusion1D_TwoSpecies": r"testval\s*=\s*([-0-9.e]+)",
    "Example115_HeterogeneousCatalysis1D": r"testval\s*=\s*([-0-9.e]+)",
    "Example160_UnipolarDriftDiffusion1D": r"evolval\s*=\s*([-0-9.e]+)",
    "Example161_BipolarDriftDiffusionCurrent": r"testval\s*=\s*([-0-9.e]+)",
    "Example207_NonlinearPoisson2D": r"testval\s*=\s*([-0-9.e]+)",
    "Example210_NonlinearPoisson2D_Reaction": r"testval\s*=\s*([-0-9.e]+)",
    "Example215_NonlinearPoisson2D_BoundaryReaction": r"testval\s*=\s*([-0-9.e]+)",
    # the value is inline in runtests: @test main(; unknown_storage = :sparse) ≈ value
    "Example220_NonlinearPoisson2D_BoundarySpecies": r"≈\s*([-0-9.e]+)",
    "Example301_Laplace3D": r"testval\s*=\s*([-0-9.e]+)",
    "Example430_ParameterDerivativesStationary": r"testval\s*=\s*([-0-9.e]+)",
    "Example440_ParallelState": r"testval\s*=\s*([-0-9.e]+)",
}


def testvals():
    out = {}
    for name, pat in EXAMPLES.items():
        rel = f"examples/{name}.jl"
        lines = open(os.path.join(REF, rel)).read().splitlines()
        for i, line in enumerate(lines, 1):
            m = re.search(pat, line)
            if m:
                out[name] = {"value": float(m.group(1)), "source": f"{rel}:{i}"}
                break
        else:
            raise RuntimeError(f"no golden value found in {rel}")
    return out


def bernoulli_kat(stride=100):
    decimal.getcontext().prec = 60
    D = decimal.Decimal

    def B(x):
        bx = D(x)
        if bx == 0:
            return 1.0
        return float(bx / (bx.exp() - 1))

    small = np.array([-1 + k * 1.00001e-5 for k in range(0, 200000, stride)])
    large = np.array([-100 + k * 1.00001e-3 for k in range(0, 200000, stride)])
    xs = np.concatenate([small, large])
    return xs, np.array([B(x) for x in xs]), np.array([B(-x) for x in xs])


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_fixtures.py /path/to/reference")
    REF = sys.argv[1]
    tv = testvals()
    with open(os.path.join(HERE, "reference_testvals.json"), "w") as f:
        json.dump(tv, f, indent=1, sort_keys=True)
    xs, bp, bm = bernoulli_kat()
    np.savez_compressed(os.path.join(HERE, "bernoulli_kat.npz"), x=xs, bp=bp, bm=bm)
    print(json.dumps(tv, indent=1), xs.size)
