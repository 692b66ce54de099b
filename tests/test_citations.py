"""Every `file:line` citation of the TimeEvolver reference in this repository
points inside the cited file, and the boundary header cites the functions it
replaces.

The line counts come from tests/golden/reference_lines.json (written by
tests/golden/make_reference_lines.py from the reference tree), so the range
check runs without the reference.  The content check of the boundary
citations reads the reference tree itself and runs only where
TE_REFERENCE_DIR names it.
"""
import glob
import json
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TABLE = os.path.join(ROOT, "tests", "golden", "reference_lines.json")
REF_DIR = os.environ.get("TE_REFERENCE_DIR")

# files of this repository whose comments cite the reference
SOURCES = ["include/*.h", "timeevolver_gb300/*.py", "timeevolver_gb300/csrc/*", "timeevolver_gb300/host/*",
           "oracle/*.py", "oracle/*.cpp", "oracle/*.h", "oracle/ref_shim/**/*", "tests/*.py", "tests/cpp/*",
           "tests/golden/*.py", "bench.py", "__graft_entry__.py"]

# path:line or path:a-b, optionally followed by ", :c-d" ranges in the same file
CITE = re.compile(r"((?:[A-Za-z_.]+/)*[A-Za-z_]+\.(?:cpp|h|hpp|yml|nb)|CMakeLists\.txt):(\d+)(?:-(\d+))?"
                  r"((?:,\s*:\d+(?:-\d+)?)*)")
MORE = re.compile(r":(\d+)(?:-(\d+))?")

# files of this repository that share a name with a reference file: a citation
# is a reference citation when it names the reference's directory
OWN_PREFIXES = ("timeevolver_gb300/", "host/", "csrc/", "include/", "oracle/", "tests/")


def _table():
    with open(TABLE) as f:
        return json.load(f)


def _resolve(name, table):
    if name in table:
        return name
    hits = [p for p in table if p == name or p.endswith("/" + name)]
    return hits[0] if len(hits) == 1 else None


def _citations():
    out = []
    for pat in SOURCES:
        for path in sorted(glob.glob(os.path.join(ROOT, pat), recursive=True)):
            if not os.path.isfile(path) or "__pycache__" in path or path.endswith(".so"):
                continue
            rel = os.path.relpath(path, ROOT)
            if rel == "tests/test_citations.py":
                continue
            with open(path, errors="replace") as f:
                for lineno, line in enumerate(f, 1):
                    for m in CITE.finditer(line):
                        name = m.group(1)
                        if name.startswith(OWN_PREFIXES):
                            continue
                        ranges = [(int(m.group(2)), int(m.group(3) or m.group(2)))]
                        ranges += [(int(a), int(b or a)) for a, b in MORE.findall(m.group(4) or "")]
                        out.append((rel, lineno, name, ranges))
    return out


def test_table_covers_the_cited_sources():
    table = _table()
    for f in ["core/krylovTimeEvolver.cpp", "core/matrixDataTypes.cpp", "core/krylovObservables.cpp",
              "helper/Basis.cpp", "helper/hamiltonian.cpp", "helper/krylovHelper.cpp"]:
        assert f in table


def test_every_reference_citation_is_inside_its_file():
    table = _table()
    cites = _citations()
    assert len(cites) > 100
    bad = []
    for rel, lineno, name, ranges in cites:
        target = _resolve(name, table)
        if target is None:
            # own files cited by name (e.g. te_oracle.cpp) are not reference citations
            if os.path.exists(os.path.join(ROOT, name)) or glob.glob(os.path.join(ROOT, "**", os.path.basename(name)),
                                                                    recursive=True):
                continue
            bad.append("%s:%d cites %s, which is not a reference file" % (rel, lineno, name))
            continue
        for a, b in ranges:
            if not (1 <= a <= b <= table[target]):
                bad.append("%s:%d cites %s:%d-%d; the file has %d lines" % (rel, lineno, target, a, b,
                                                                          table[target]))
    assert not bad, "\n".join(bad)


# boundary entries of include/tegpu.h and the reference text their ranges must contain
BOUNDARY = [
    ("core/matrixDataTypes.cpp", 169, 190, "smatrix::spMV"),
    ("core/matrixDataTypes.cpp", 196, 240, "smatrix::initialize"),
    ("core/matrixDataTypes.cpp", 67, 79, "smatrix::norm1"),
    ("core/matrixDataTypes.cpp", 108, 134, "smatrix::smatrix("),
    ("core/krylovObservables.cpp", 180, 184, "Incompatible dimensions"),
    ("core/krylovObservables.cpp", 173, 236, "krylovVectorObservable::expectation"),
    ("core/krylovTimeEvolver.cpp", 261, 512, "krylovTimeEvolver::timeEvolve"),
    ("core/krylovTimeEvolver.cpp", 662, 676, "krylovTimeEvolver::generateReturn"),
    ("core/krylovTimeEvolver.cpp", 26, 94, "krylovTimeEvolver::krylovTimeEvolver"),
    ("core/krylovTimeEvolver.cpp", 39, 43, "Hsize == 0"),
    ("core/krylovTimeEvolver.cpp", 45, 48, "cblas_dznrm2"),
    ("core/krylovTimeEvolver.cpp", 203, 207, "GO_MAX"),
    ("core/krylovTimeEvolver.cpp", 537, 546, "cblas_zaxpy"),
    ("core/krylovTimeEvolver.cpp", 665, 665, "evolvedState"),
    ("core/krylovTimeEvolver.h", 59, 60, "krylovTimeEvolver("),
    ("core/krylovTimeEvolver.h", 61, 61, "timeEvolve"),
    ("core/krylovTimeEvolver.h", 32, 51, "krylovReturn"),
    ("core/krylovObservables.h", 42, 42, "expectation"),
]


def test_boundary_header_cites_these_ranges():
    with open(os.path.join(ROOT, "include", "tegpu.h")) as f:
        header = f.read()
    for path, a, b, _ in BOUNDARY:
        short = os.path.basename(path)
        span = "%d-%d" % (a, b) if a != b else "%d" % a
        assert (":" + span) in header and short in header, (path, span)


@pytest.mark.skipif(not REF_DIR, reason="TE_REFERENCE_DIR not set (reference tree absent)")
def test_boundary_ranges_contain_the_replaced_code():
    for path, a, b, text in BOUNDARY:
        with open(os.path.join(REF_DIR, path), errors="replace") as f:
            lines = f.read().split("\n")
        assert any(text in ln for ln in lines[a - 1:b]), "%s:%d-%d does not contain %r" % (path, a, b, text)


@pytest.mark.skipif(not REF_DIR, reason="TE_REFERENCE_DIR not set (reference tree absent)")
def test_line_table_matches_the_reference_tree():
    table = _table()
    for rel, n in table.items():
        with open(os.path.join(REF_DIR, rel), "rb") as f:
            data = f.read()
        assert data.count(b"\n") + (0 if data.endswith(b"\n") or not data else 1) == n, rel
