"""Regenerates tests/golden/ref_tables.json from the reference's own table code.

Run where the reference sources are (argument, else $GBNTT_REFERENCE_ROOT,
else `reference` beside this repository):

    python tests/golden/make_golden.py [REF_DIR]

It builds oracle/_ref/ref_tables (the reference's src/twiddle.h and
src/auxiliary.h compiled against oracle/ref_stub/adf.h, recipe in
oracle/Makefile), runs it, and stores for every table its length, the SHA-256
of its values written as decimal text separated by single spaces, and the
values themselves when the table has at most 512 entries.  The tests compare
the oracle's tables and the GPU library's tables against this file; nothing at
test time needs the reference sources.
"""
import hashlib
import json
import os
import subprocess
import sys


def default_reference_root():
    repo = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    return os.environ.get("GBNTT_REFERENCE_ROOT") or os.path.join(os.path.dirname(repo), "reference")

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def table_hash(values):
    return hashlib.sha256(" ".join(str(int(v)) for v in values).encode()).hexdigest()


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else default_reference_root()
    oracle = os.path.join(ROOT, "oracle")
    subprocess.run(["make", "-s", "-C", oracle, "ref", f"REF={ref}"], check=True)
    out = subprocess.run([os.path.join(oracle, "_ref", "ref_tables")], check=True,
                         capture_output=True, text=True).stdout
    tables = {}
    for line in out.splitlines():
        head, _, body = line.partition(":")
        fam, n, q, root, which, layer, length = head.split()
        vals = [int(v) for v in body.split()]
        assert len(vals) == int(length)
        key = f"{fam} {n} {q} {root} {which} {layer}"
        entry = {"len": len(vals), "sha256": table_hash(vals)}
        if len(vals) <= 512:
            entry["values"] = vals
        tables[key] = entry
    doc = {
        "source": "reference src/twiddle.h + src/auxiliary.h built with oracle/ref_stub/adf.h",
        "hash": "sha256 of the decimal values joined by single spaces",
        "tables": tables,
    }
    with open(os.path.join(HERE, "ref_tables.json"), "w") as f:
        json.dump(doc, f, indent=0, sort_keys=True)
    print(f"wrote {len(tables)} tables")


if __name__ == "__main__":
    main()
