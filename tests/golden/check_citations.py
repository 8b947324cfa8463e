"""Checks that every citation of a reference file with line numbers (``src/…jl:N``,
``src/…jl:N-M``, ``examples/…jl:N``, ``test/…jl:N``) in this repository's sources and documents
points inside the cited file, and that the cited file exists.

Scanned: the package, the oracle, the tests, the C header, the top-level Python files and the
repository's own user-facing documents (DOCS below); other documents at the top level are
not part of the product and are not scanned.  The reference tree is read from the first argument,
else from $HDG_REFERENCE_TREE, else from the reference checkout of the build machine.
Usage:  python tests/golden/check_citations.py [reference-tree]
Prints one line per bad citation and exits 1 if there is any.
"""
from __future__ import annotations

import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CITE = re.compile(r"((?:src|examples|test)/[A-Za-z0-9_./]+?\.jl):(\d+)(?:\s*[-–]\s*(\d+))?((?:\s*,\s*:?\d+(?:\s*[-–]\s*\d+)?)*)")
MORE = re.compile(r":?(\d+)(?:\s*[-–]\s*(\d+))?")
SKIP_DIRS = {"_build", "__pycache__", ".pytest_cache"}
EXTS = (".py", ".cpp", ".cu", ".cuh", ".h", ".md")
SOURCE_DIRS = ("hdiscontinuousgalerkin.jl_gb300", "oracle", "tests", "include", "profiles")
DOCS = ("DESIGN.md", "INTEGRATION.md", "README.md")


def reference_tree(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    for cand in (argv[0] if argv else None, os.environ.get("HDG_REFERENCE_TREE"), "/root/reference"):
        if cand and os.path.isdir(cand):
            return cand
    return None


def scanned_files():
    for top in SOURCE_DIRS:
        for d, dirs, files in os.walk(os.path.join(ROOT, top)):
            dirs[:] = [x for x in dirs if x not in SKIP_DIRS]
            for fn in files:
                if fn.endswith(EXTS):
                    yield os.path.join(d, fn)
    for fn in sorted(os.listdir(ROOT)):
        if fn.endswith(".py") or fn in DOCS:
            yield os.path.join(ROOT, fn)


def citations():
    for path in scanned_files():
        if os.path.isfile(path):
            with open(path, encoding="utf-8", errors="replace") as fh:
                for ln, text in enumerate(fh, 1):
                    for m in CITE.finditer(text):
                        ranges = [(int(m.group(2)), int(m.group(3) or m.group(2)))]
                        for mm in MORE.finditer(m.group(4) or ""):
                            ranges.append((int(mm.group(1)), int(mm.group(2) or mm.group(1))))
                        yield os.path.relpath(path, ROOT), ln, m.group(1), ranges


def check(tree):
    lengths, bad, n = {}, [], 0
    for where, ln, cited, ranges in citations():
        n += 1
        full = os.path.join(tree, cited)
        if cited not in lengths:
            lengths[cited] = sum(1 for _ in open(full, encoding="utf-8", errors="replace")) if os.path.isfile(full) else -1
        L = lengths[cited]
        for a, b in ranges:
            if L < 0 or a < 1 or b < a or b > L:
                bad.append(f"{where}:{ln}: {cited}:{a}-{b} (file has {L} lines)" if L >= 0 else
                           f"{where}:{ln}: {cited} does not exist")
    return n, bad


if __name__ == "__main__":
    tree = reference_tree()
    if not tree:
        sys.exit("reference tree not found")
    n, bad = check(tree)
    print("\n".join(bad))
    print(f"{n} citations, {len(bad)} out of range")
    sys.exit(1 if bad else 0)
