"""Every reference citation of the form dir/file.f:LINE or dir/file.f:FIRST-LAST in the
header, the library's sources and the oracle names a file of the reference tree
($SDE_REFERENCE, else /root/reference) and lines inside it.  Skipped where the tree is
absent."""
import glob
import os
import re

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REF = os.environ.get("SDE_REFERENCE") or "/root/reference"

CITE = re.compile(r'\b((?:source/)?[a-z][a-z0-9]*/[a-z0-9_]+\.(?:f|c|h|inc))\s*:\s*(\d+)(?:\s*-\s*(\d+))?')


def _sources():
    pats = ("include/*.h", "sde_gb300/csrc/*.cu", "sde_gb300/csrc/*.cuh", "sde_gb300/*.py",
            "oracle/*.c", "oracle/*.h", "oracle/*.py")
    out = []
    for p in pats:
        out += glob.glob(os.path.join(ROOT, p))
    return sorted(out)


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "source")), reason="reference tree not present")
def test_reference_citations_land_inside_their_files():
    lines = {}
    bad, n = [], 0
    for f in _sources():
        text = open(f, encoding="utf-8", errors="replace").read()
        for m in CITE.finditer(text):
            path, first, last = m.group(1), int(m.group(2)), m.group(3)
            last = int(last) if last else first
            cands = [os.path.join(REF, path), os.path.join(REF, "source", path)]
            p = next((c for c in cands if os.path.isfile(c)), None)
            n += 1
            if p is None:
                bad.append("%s: %s (no such file)" % (os.path.relpath(f, ROOT), m.group(0)))
                continue
            if p not in lines:
                with open(p, errors="replace") as fh:
                    lines[p] = sum(1 for _ in fh)
            if first < 1 or last < first or last > lines[p]:
                bad.append("%s: %s (file has %d lines)" % (os.path.relpath(f, ROOT), m.group(0), lines[p]))
    assert n > 100
    assert not bad, "\n".join(bad)
