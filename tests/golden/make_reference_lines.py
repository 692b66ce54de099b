"""Write reference_lines.json: the line count of every source and text file of
the TimeEvolver reference tree, keyed by its path inside the project.

The citation test (tests/test_citations.py) checks every `file:line` citation
of this repository against this table, so that it runs where the reference
tree is absent.  Usage: python make_reference_lines.py [REFERENCE_DIR]
(default: $TE_REFERENCE_DIR).
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
EXTS = (".cpp", ".h", ".hpp", ".txt", ".md", ".yml", ".nb", ".py", ".csv")


def main(ref_root):
    table = {}
    for dp, dn, fn in os.walk(ref_root):
        dn[:] = sorted(d for d in dn if d != ".git")
        for f in sorted(fn):
            if not f.endswith(EXTS) and f != "CMakeLists.txt":
                continue
            p = os.path.join(dp, f)
            with open(p, "rb") as fh:
                data = fh.read()
            table[os.path.relpath(p, ref_root)] = data.count(b"\n") + (0 if data.endswith(b"\n") or not data else 1)
    with open(os.path.join(HERE, "reference_lines.json"), "w") as fh:
        json.dump(table, fh, indent=1, sort_keys=True)
        fh.write("\n")


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("TE_REFERENCE_DIR")
    if not root:
        sys.exit("usage: make_reference_lines.py REFERENCE_DIR (or set TE_REFERENCE_DIR)")
    main(root)
