"""Regenerate gbneck_tables.h, the GBneck model's parameter tables.

The GBneck (gb=7) and GBneck2 (gb=8) descreening models use two published
21x21 lookup tables -- the separation at which the "neck" integral peaks and
its peak value (already divided by 4*pi) -- indexed by the two atoms' intrinsic
radii in 0.05 A steps from 1.0 to 2.0 A, plus the per-element GBneck2
constants.  These numbers are model parameters and must be bit-identical to
the reference's (src/sff/gbneck.h:7-170), so this script extracts them from
that header and writes them into flat arrays of our own layout.

Usage (where the reference's source tree is at hand):
    python nabc_gb300/csrc/gen_neck_tables.py <reference tree>/src/sff/gbneck.h
"""
import os
import re
import sys


def extract_table(text, name):
    start = text.index(name)
    body = text[text.index("{", start):text.index("};", start)]
    vals = re.findall(r"[-+]?\d+\.\d+(?:[eE][-+]?\d+)?", body)
    if len(vals) != 441:
        raise SystemExit(f"{name}: expected 441 values, found {len(vals)}")
    return vals


def main():
    src = sys.argv[1]
    text = open(src).read()
    pos = extract_table(text, "neckMaxPos[21][21]")
    val = extract_table(text, "neckMaxVal[21][21]")
    consts = dict(re.findall(r"#define\s+(GB8_\w+)\s+([-+]?\d+\.?\d*)", text))
    neckcut = re.search(r"GBNECKCUT\s*=\s*([\d.]+)", text).group(1)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "gbneck_tables.h")
    with open(out, "w") as f:
        f.write("/* Generated by gen_neck_tables.py: GBneck model parameters (published\n"
                " * tables; must equal the reference's src/sff/gbneck.h).  Row-major\n"
                " * [idx_i*21 + idx_j], idx = (int)((rborn - 1.0)*20 + 0.5). */\n")
        f.write("#ifndef SFFG_GBNECK_TABLES_H\n#define SFFG_GBNECK_TABLES_H\n\n")
        f.write(f"#define SFFG_GBNECK_CUT {neckcut}\n")
        for k in sorted(consts):
            f.write(f"#define SFFG_{k} {consts[k]}\n")
        for name, vals in (("sffg_neck_max_pos", pos), ("sffg_neck_max_val", val)):
            f.write(f"\nstatic const double {name}[441] = {{\n")
            for i in range(0, 441, 7):
                f.write("  " + ", ".join(vals[i:i + 7]) + ",\n")
            f.write("};\n")
        f.write("\n#endif\n")
    print("wrote", out)


if __name__ == "__main__":
    main()
