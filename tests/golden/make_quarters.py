"""Cuts the reference's harness input files down to small quarter-file fixtures.

The reference ships ramp inputs for its harness as four quarter streams
(data/input_data_q{0..3}.txt with 8 int16 values per line, data_int32/ with 4
int32 values per line).  This script keeps the first POLYS polynomials' worth
of each stream (n = 4096 for the int16 designs, 2048 for the int32 designs,
the lengths of src/project.cpp:139-157) under tests/golden/quarters/, so the
tests can run the harness format without the reference tree.

    python tests/golden/make_quarters.py [reference root]

(default: $GBNTT_REFERENCE_ROOT, else `reference` beside this repository)
"""
import os
import sys


def default_reference_root():
    repo = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    return os.environ.get("GBNTT_REFERENCE_ROOT") or os.path.join(os.path.dirname(repo), "reference")

POLYS = 4
HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref):
    for sub, n, per_line in (("data", 4096, 8), ("data_int32", 2048, 4)):
        keep_lines = POLYS * (n // 4) // per_line
        dst = os.path.join(HERE, "quarters", sub)
        os.makedirs(dst, exist_ok=True)
        for k in range(4):
            name = f"input_data_q{k}.txt"
            with open(os.path.join(ref, sub, name)) as f:
                lines = [next(f) for _ in range(keep_lines)]
            with open(os.path.join(dst, name), "w") as f:
                f.writelines(lines)
        print(f"{sub}: {POLYS} polynomials of n = {n} ({keep_lines} lines per quarter file)")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else default_reference_root())
