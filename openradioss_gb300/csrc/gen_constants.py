"""Generate rg_constants.h: the numeric constants of the explicit hot path.

The reference defines its constants as chained ``my_real`` parameter
expressions (common_source/modules/constant_mod.F:579-1030), e.g.
``ONEP333 = ONEP33 + THREEEM3`` (1.333, not 4/3) and ``ZEP9``-style decimals
built from integer ratios.  Reproducing them bit-for-bit needs the same
evaluation order in IEEE double, so this script evaluates every parameter of
that module in declaration order with Python floats (IEEE binary64,
round-to-nearest, left-to-right like Fortran) and writes the values used by
the kernels and the oracle as exact hexadecimal literals.

Run from the repository root with the reference checked out:
    python openradioss_gb300/csrc/gen_constants.py <path-to-reference>
The generated header is committed; nothing at build or run time reads the
reference.
"""
import math
import os
import re
import sys

WANTED = [
    "ZERO", "ONE", "TWO", "THREE", "FOUR", "EIGHT", "TEN", "HUNDRED", "HALF",
    "THIRD", "FOURTH", "ONE_OVER_8", "ONE_OVER_64", "TWO_THIRD", "THREE_HALF",
    "ONEP333", "ONEP1", "ZEP9", "EM01", "EM03", "EM06", "EM10", "EM15", "EM20",
    "EM30", "EP02", "EP06", "EP20", "EP30", "ZEP499", "FOUR_OVER_3",
    "FIVE", "SIX", "TWELVE", "ONE_OVER_6", "ONE_OVER_12", "EM04", "EP03",
    "ZEP81", "ZEP072169", "ONEP414", "ONE_OVER_9", "THREE_OVER_4",
    "FOUR_OVER_5", "EM07", "NINE", "ONEP00001",
]


def evaluate(path):
    env = {}
    pat = re.compile(r"^\s*my_real\s*,\s*parameter\s*::\s*(\w+)\s*=\s*(.+?)\s*$",
                     re.IGNORECASE)
    for line in open(path):
        m = pat.match(line)
        if not m:
            continue
        name, expr = m.group(1).upper(), m.group(2)
        expr = expr.split("!")[0]
        # Fortran literals of the form "1." / "1E20" -> python floats.  All
        # literals in the module are integers or powers of ten, exact in both
        # single and double precision.
        expr = re.sub(r"(\d+)\.(?!\d)", r"\1.0", expr)
        funcs = {"SQRT": "math.sqrt", "ATAN2": "math.atan2"}
        pyexpr = re.sub(r"\b([A-Za-z_]\w*)\b",
                        lambda t: funcs.get(t.group(1).upper(),
                                            "env['%s']" % t.group(1).upper()),
                        expr)
        env[name] = float(eval(pyexpr, {"env": env, "math": math}))
    return env


def main():
    # root of the OpenRadioss source tree: first argument or OPENRADIOSS_SRC
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("OPENRADIOSS_SRC")
    if not ref:
        sys.exit("usage: gen_constants.py <root of the OpenRadioss source tree> "
                 "(or set OPENRADIOSS_SRC)")
    env = evaluate(ref + "/common_source/modules/constant_mod.F")
    out = [
        "// Generated by gen_constants.py from the reference's constant module",
        "// (common_source/modules/constant_mod.F).  Exact IEEE-754 binary64",
        "// values of the chained parameter expressions; do not edit by hand.",
        "#pragma once",
        "",
    ]
    for n in WANTED:
        v = env[n]
        out.append("#define RG_%-12s (%s) /* %.17g */" % (n, v.hex(), v))
    # 1.1 in RESOL's "DT2 = MIN(DT2, 1.1*DT2OLD, DTMX)" is a default-real
    # (single precision) literal promoted to double (engine/source/engine/resol.F:6352).
    import struct
    f11 = struct.unpack("f", struct.pack("f", 1.1))[0]
    out.append("#define RG_%-12s (%s) /* %.17g: REAL*4 literal 1.1 */" % (
        "SP_1P1", f11.hex(), f11))
    open("openradioss_gb300/csrc/rg_constants.h", "w").write("\n".join(out) + "\n")


if __name__ == "__main__":
    main()
