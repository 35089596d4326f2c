"""Every reference citation in the sources (``path/file.jl:a-b``) names one file of the
reference and lines that exist in it; where the citing line names a reference function,
the cited lines contain that name (CPU).

The reference checkout is not shipped with this repository: set MCX_REFERENCE_ROOT to the
MonteCarloX.jl checkout to run these tests; without it they are skipped."""
import os

import pytest

import citations as C

REF = os.environ.get("MCX_REFERENCE_ROOT")
pytestmark = pytest.mark.skipif(not REF or not os.path.isdir(REF or ""),
                                reason="set MCX_REFERENCE_ROOT to the reference checkout")

# reference names whose citation should contain them (checked when the citing line names
# exactly one of them)
NAMES = ["spin_flip!", "accept!", "init!", "flip_changes", "local_pair_interactions", "logistic", "set_betas",
         "exchange_log_ratio", "record_visit!", "pick_site", "_propose_state", "propose_changes", "local_coupling",
         "merge_histograms!", "distribute_logweight!", "log_sum", "distribution_from_logdos",
         "optimize_exchange_interval!", "attempt_exchange_pair!", "restore_checkpoint", "acceptance_rate",
         "with_parallel", "_accept_exchange", "_binindex", "_check_symmetric", "run_chain!"]


def _all():
    files = C.reference_files(REF)
    out = []
    for f in C.source_files():
        for no, suf, a, b in C.citations(f):
            out.append((os.path.relpath(f, C.ROOT), no, suf, a, b, files))
    return out


def test_every_citation_resolves_to_existing_lines():
    bad = []
    for src, no, suf, a, b, files in _all():
        r = C.resolve(suf, files)
        if len(r) != 1:
            bad.append("%s:%d %s matches %s" % (src, no, suf, r))
        elif not (1 <= a <= b <= files[r[0]]):
            bad.append("%s:%d %s:%d-%d beyond %d lines" % (src, no, r[0], a, b, files[r[0]]))
    assert not bad, "\n".join(bad)


def test_named_functions_are_in_the_cited_lines():
    bad = []
    cache = {}
    lines = {}
    for src, no, suf, a, b, files in _all():
        path = C.resolve(suf, files)[0]
        if path not in cache:
            cache[path] = open(os.path.join(REF, path), encoding="utf-8", errors="replace").read().split("\n")
        lines.setdefault((src, no), []).append((path, a, b, "\n".join(cache[path][a - 1:b])))
    for (src, no), cites in lines.items():
        line = open(os.path.join(C.ROOT, src), encoding="utf-8").read().split("\n")[no - 1]
        named = [n for n in NAMES if n in line]
        if len(named) != 1:
            continue
        if not any(named[0] in text for _, _, _, text in cites):
            bad.append("%s:%d cites %s for %s" % (src, no, ["%s:%d-%d" % c[:3] for c in cites], named[0]))
    assert not bad, "\n".join(bad)
