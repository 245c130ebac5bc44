#!/usr/bin/env python3
"""Writes csrc/moduli_sets.h from the reference's predefined moduli sets.

The reference selects its moduli set at compile time by replacing src/params.h
with one of src/params/32-bit-moduli/params.<N>_32bit.h (README.md:48-52); each
file defines RNS_MODULI_SIZE, RNS_MODULI_PRODUCT_LOG2, RNS_P2_SCALING_THRESHOLD,
RNS_EVAL_RELATIVE_ERROR and RNS_MODULI_VALUES.  This script copies those values,
unchanged, into one C header so that the library can hold several sets at once.

Run it where the reference checkout exists:
    python gen_moduli_sets.py <path to the reference checkout>/src
The generated header is committed; the build never runs this script.
"""
import pathlib
import re
import sys

HERE = pathlib.Path(__file__).resolve().parent


def parse(path):
    text = path.read_text()
    text = re.sub(r"\\\n", " ", text)

    def grab(name):
        m = re.search(r"#define\s+%s\s+\(?\s*([^)\n]+?)\s*\)?\s*$" % name, text, re.M)
        return m.group(1).strip()

    size = int(grab("RNS_MODULI_SIZE"))
    log2 = int(grab("RNS_MODULI_PRODUCT_LOG2"))
    thr = int(grab("RNS_P2_SCALING_THRESHOLD"))
    rel = grab("RNS_EVAL_RELATIVE_ERROR")
    vals = re.search(r"#define\s+RNS_MODULI_VALUES\s*\{([^}]*)\}", text).group(1)
    moduli = [int(v) for v in vals.replace(" ", "").split(",") if v]
    assert len(moduli) == size, path
    assert thr == 30, path
    return size, log2, rel, moduli


def main():
    if len(sys.argv) < 2:
        sys.exit("usage: gen_moduli_sets.py <reference src/ directory>")
    src = pathlib.Path(sys.argv[1])
    sets = []
    for p in sorted((src / "params" / "32-bit-moduli").glob("params.*_32bit.h"),
                    key=lambda p: int(p.name.split(".")[1].split("_")[0])):
        sets.append((p, *parse(p)))
    out = [
        "/*",
        " * Predefined moduli sets of 32-bit RNS moduli, copied value for value from the",
        " * reference's src/params/32-bit-moduli/params.<N>_32bit.h by gen_moduli_sets.py.",
        " * Every set uses RNS_P2_SCALING_THRESHOLD = 30 and RNS_EVAL_RELATIVE_ERROR = 1e-7.",
        " */",
        "#ifndef MPRES_MODULI_SETS_H",
        "#define MPRES_MODULI_SETS_H",
        "",
        "#define MPRES_P2_SCALING_THRESHOLD 30",
        "#define MPRES_EVAL_RELATIVE_ERROR 0.0000001",
        "",
    ]
    for p, size, log2, rel, moduli in sets:
        assert float(rel) == 1e-7, p
        out.append("/* params/32-bit-moduli/%s */" % p.name)
        out.append("#define MPRES_SET%d_LOG2 %d" % (size, log2))
        rows = []
        for i in range(0, size, 8):
            rows.append("    " + ", ".join(str(v) for v in moduli[i:i + 8]))
        out.append("#define MPRES_SET%d_MODULI { \\" % size)
        out.append(", \\\n".join(rows) + " }")
        out.append("")
    out.append("#endif")
    (HERE / "csrc" / "moduli_sets.h").write_text("\n".join(out) + "\n")
    print("wrote %d sets" % len(sets))


if __name__ == "__main__":
    main()
