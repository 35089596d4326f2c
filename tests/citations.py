"""Extraction of the reference citations (``path/file.jl:a-b``) written in the sources.

A citation names a Julia file of MonteCarloX.jl by a path suffix (``ising.jl``,
``src/algorithms/metropolis.jl``, ``SpinSystems/src/ising.jl``) and a line or a range;
``, :c-d`` or ``, c-d`` after it, and a bare ``:c-d`` later on, cite more lines of the
file named last.  Used by tests/test_citations.py.
"""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SOURCES = ["include", "oracle", "montecarlox.jl_gb300/csrc", "montecarlox.jl_gb300/mcx", "tests"]
SOURCE_FILES = ["bench.py", "__graft_entry__.py", "DESIGN.md", "INTEGRATION.md", "README.md"]
EXTS = (".h", ".c", ".cu", ".cuh", ".py", ".md")

_FILE = re.compile(r"((?:[A-Za-z0-9_.]+/)*[A-Za-z0-9_]+\.jl)((?::\d+(?:-\d+)?)(?:,\s*:?\d+(?:-\d+)?)*)")
_BARE = re.compile(r"(?<![\w./\-\[:]):(\d+)(?:-(\d+))?(?![\w.\]:])")
_RANGE = re.compile(r":?(\d+)(?:-(\d+))?")


def source_files():
    out = []
    for d in SOURCES:
        base = os.path.join(ROOT, d)
        for dirpath, _, names in os.walk(base):
            if "_build" in dirpath or "_ref" in dirpath or "__pycache__" in dirpath or "/lib" in dirpath:
                continue
            for n in sorted(names):
                if n.endswith(EXTS) and n not in ("citations.py", "test_citations.py"):
                    out.append(os.path.join(dirpath, n))
    out += [os.path.join(ROOT, f) for f in SOURCE_FILES if os.path.exists(os.path.join(ROOT, f))]
    return out


def citations(path):
    """(source line number, cited path suffix, first line, last line) for every citation."""
    out = []
    last = None
    for no, line in enumerate(open(path, encoding="utf-8", errors="replace"), 1):
        toks = [(m.start(), m.end(), m) for m in _FILE.finditer(line)]
        spans = [(s, e) for s, e, _ in toks]
        toks += [(m.start(), m.end(), m) for m in _BARE.finditer(line)
                 if not any(s <= m.start() < e for s, e in spans)]
        for _, _, m in sorted(toks, key=lambda t: t[0]):
            if m.re is _FILE:
                last = m.group(1)
                for r in _RANGE.finditer(m.group(2)):
                    a = int(r.group(1))
                    out.append((no, last, a, int(r.group(2)) if r.group(2) else a))
            elif last is not None:
                a = int(m.group(1))
                out.append((no, last, a, int(m.group(2)) if m.group(2) else a))
    return out


def reference_files(root):
    files = {}
    for dirpath, _, names in os.walk(root):
        if "/.git" in dirpath:
            continue
        for n in names:
            if n.endswith(".jl"):
                p = os.path.join(dirpath, n)
                files[os.path.relpath(p, root)] = sum(1 for _ in open(p, encoding="utf-8", errors="replace"))
    return files


def resolve(suffix, files):
    """Reference paths whose path ends with the cited suffix."""
    return [p for p in files if p == suffix or p.endswith("/" + suffix)]
