"""Generate the golden fixtures of tests/golden/ (run once, in the build
container; the fixtures are committed and nothing reads the reference at
test time).

Sources:
  * the reference's own known-answer inputs, read as TEXT from
    GenericLinearAlgebra.jl test/eigenselfadjoint.jl: the issue-123 4x4
    BigFloat matrix (:125-131) and the 2x2 eig2x2! (d, e) table (:135-149);
  * seeded GOE matrices and a seeded SymTridiagonal, solved by the 256-bit
    mpmath restatement of the reference algorithm (oracle/gla_ref_mp.py), the
    stand-in for running the reference on BigFloat.
"""
import argparse
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import gla_ref_mp as MP  # noqa: E402

REF_TEST_REL = os.path.join("test", "eigenselfadjoint.jl")
DIGITS = 75
LARGE_CASES = [(64, 1), (128, 7)]


def s(x):
    import mpmath
    return mpmath.nstr(x, DIGITS, strip_zeros=False)


def parse_issue123(text):
    block = text[text.index('@testset "issue 123"'):]
    block = block[: block.index("F = eigen(M)")]
    vals = re.findall(r'big"([-0-9.eE+]+)"', block)
    assert len(vals) == 16, len(vals)
    return [vals[4 * i: 4 * i + 4] for i in range(4)]


def parse_2x2(text):
    block = text[text.index("2x2 cases"):]
    block = block[: block.index("V = Matrix")]
    cases = re.findall(r"\(\[([^\]]*)\],\s*\[([^\]]*)\]\)", block)
    out = []
    for d, e in cases:
        out.append(([float(v) for v in d.split(",")], [float(v) for v in e.split(",")]))
    assert len(out) == 9, len(out)
    return out


def goe(n, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    B = rng.standard_normal((n, n))
    return (B + B.T) / 2


def main_large():
    out = {"source": "256-bit restatement of GenericLinearAlgebra.jl v0.4.0 eigen!(Hermitian) "
                     "(oracle/gla_ref_mp.py) on seeded GOE matrices",
           "precision_bits": MP.PREC, "goe": []}
    for n, seed in LARGE_CASES:
        A = goe(n, seed)
        w, V = MP.syev(A.tolist(), "V")
        out["goe"].append({"n": n, "seed": seed, "A": [[float(v).hex() for v in row] for row in A],
                           "w": [s(x) for x in w], "V": [[float(x) for x in row] for row in V]})
        print("goe", n, "done", flush=True)
    with open(os.path.join(HERE, "golden_large.json"), "w") as f:
        json.dump(out, f)
    print("wrote", os.path.join(HERE, "golden_large.json"))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("GLA_REFERENCE", ""),
                    help="GenericLinearAlgebra.jl checkout (read as text only)")
    ap.add_argument("--large", action="store_true", help="write golden_large.json instead")
    args = ap.parse_args()
    if args.large:
        main_large()
        return
    if not args.reference:
        ap.error("name the reference checkout with --reference or GLA_REFERENCE")
    text = open(os.path.join(args.reference, REF_TEST_REL)).read()
    out = {"source": "GenericLinearAlgebra.jl v0.4.0 test/eigenselfadjoint.jl + 256-bit restatement",
           "precision_bits": MP.PREC}
    M = parse_issue123(text)
    w, V = MP.syev(M, "V")
    out["issue123"] = {"A": M, "w": [s(x) for x in w], "V": [[s(x) for x in row] for row in V]}
    out["eig2x2_cases"] = [{"d": d, "e": e} for d, e in parse_2x2(text)]
    goes = []
    for n, seed in [(3, 11), (5, 12), (8, 13), (16, 14), (24, 15)]:
        A = goe(n, seed)
        w, V = MP.syev(A.tolist(), "V")
        goes.append({"n": n, "seed": seed, "A": [[float(v).hex() for v in row] for row in A],
                     "w": [s(x) for x in w], "V": [[float(x) for x in row] for row in V]})
        print("goe", n, "done", flush=True)
    out["goe"] = goes
    # SymTridiagonal (test/eigenselfadjoint.jl:5-32 uses n = 50 BigFloat randn)
    rng = np.random.Generator(np.random.PCG64(16))
    n = 50
    dv = rng.standard_normal(n)
    ev = rng.standard_normal(n - 1)
    import mpmath
    ctx = MP._ctx()
    d = [ctx.mpf(float(v)) for v in dv]
    e = [ctx.mpf(float(v)) for v in ev]
    V = [[ctx.mpf(1) if i == j else ctx.mpf(0) for j in range(n)] for i in range(n)]
    MP.eig_ql(ctx, d, e, V, MP.eps(ctx))
    order = sorted(range(n), key=lambda i: d[i])
    out["symtridiagonal"] = {"n": n, "seed": 16, "dv": [float(v).hex() for v in dv],
                             "ev": [float(v).hex() for v in ev], "w": [s(d[i]) for i in order],
                             "V": [[float(V[r][i]) for i in order] for r in range(n)]}
    d2 = [ctx.mpf(float(v)) for v in dv]
    e2 = [ctx.mpf(float(v)) for v in ev]
    MP.eigvals_pwk(ctx, d2, e2, MP.eps(ctx))
    out["symtridiagonal"]["w_pwk"] = [s(x) for x in sorted(d2)]
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", os.path.join(HERE, "golden.json"))


if __name__ == "__main__":
    main()
