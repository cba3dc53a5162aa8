"""Every `<file>.f:N` / `<file>.f:N-M` citation of the reference's Fortran in
the library, its header, the oracle, the tests and the design notes points
at lines that exist.

REF_LINES holds the line count of each Fortran file of the reference
(Delta-function/cliffs-src); where the checkout is present the table itself
is checked against it.  Several files share a base name (errhandle.f in three
directories, opennc4feed.f in two); a citation by base name must fit the
shortest of them.
"""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

REF_LINES = {
    "MasterGrid.f": 127, "NestedGrid.f": 148, "allabout.f": 97, "apply_initial_conditions.f": 70,
    "cliffs.f": 346, "cliffs_main.f": 401, "errhandle.f": 8, "feed_children_grid.f": 181,
    "get_boundary_feed.f": 170, "get_initial_state.f": 165, "global_modules.f": 55,
    "opennc4feed.f": 87, "opennc4gages.f": 86, "opennc4max.f": 71, "opennc4sea.f": 90,
    "output_feed.f": 24, "output_gages.f": 51, "output_maxwave.f": 29, "output_sea_state.f": 66,
    "cmpboundary/InterpolateOntoBndr.f": 40, "cmpboundary/ReadGridLattice.f": 55,
    "cmpboundary/ReadSeaLattice.f": 66, "cmpboundary/cmpboundary.f": 218,
    "cmpboundary/errhandle.f": 8, "cmpboundary/get_sea_state.f": 36, "cmpboundary/opennc4feed.f": 87,
    "cmpboundary/output_bndr.f": 23, "cmpboundary/scan4wave.f": 51, "depth_ssl/depth_ssl.f": 362,
    "depth_ssl/errhandle.f": 8,
}

CITE = re.compile(r"([A-Za-z0-9_/]+\.f):(\d+)(?:-(\d+))?((?:,\s*\d+(?:-\d+)?)*)")
SCANNED = ["include", "cliffs-src_gb300", "oracle", "tests", "bench.py", "__graft_entry__.py",
           "DESIGN.md", "INTEGRATION.md", "README.md"]
EXT = (".h", ".c", ".cu", ".cuh", ".py", ".cpp", ".hpp", ".md")


def _files():
    for s in SCANNED:
        p = os.path.join(ROOT, s)
        if os.path.isfile(p):
            yield p
            continue
        for dp, dn, fn in os.walk(p):
            dn[:] = [d for d in dn if d not in ("_lib", "__pycache__", "golden")]
            for f in fn:
                if f.endswith(EXT) and f != os.path.basename(__file__):
                    yield os.path.join(dp, f)


def _length(name):
    if name in REF_LINES:
        return REF_LINES[name]
    base = os.path.basename(name)
    cands = [n for n, L in REF_LINES.items() if os.path.basename(n) == base]
    return min(REF_LINES[n] for n in cands) if cands else None


def citations():
    out = []
    for p in _files():
        with open(p, errors="replace") as f:
            for ln, line in enumerate(f, 1):
                for m in CITE.finditer(line):
                    nums = [int(m.group(2))] + ([int(m.group(3))] if m.group(3) else [])
                    nums += [int(x) for x in re.findall(r"\d+", m.group(4) or "")]
                    out.append((os.path.relpath(p, ROOT), ln, m.group(1), nums, m.group(0)))
    return out


def test_citations_point_at_existing_lines():
    cites = citations()
    assert len(cites) > 200  # the scan does see the library's citations
    bad = []
    for path, ln, name, nums, text in cites:
        L = _length(name)
        if L is None:
            bad.append(f"{path}:{ln}: {text}: no such reference file")
        elif max(nums) > L or min(nums) < 1:
            bad.append(f"{path}:{ln}: {text}: {name} has {L} lines")
        elif len(nums) >= 2 and nums[1] < nums[0]:
            bad.append(f"{path}:{ln}: {text}: range ends before it starts")
    assert not bad, "\n".join(bad)


def test_line_table_matches_checkout(reference_dir):
    seen = {}
    for dp, dn, fn in os.walk(reference_dir):
        for f in fn:
            if f.endswith(".f"):
                p = os.path.join(dp, f)
                with open(p, "rb") as fh:  # newline count, as wc -l
                    seen[os.path.relpath(p, reference_dir)] = fh.read().count(b"\n")
    assert seen == REF_LINES


@pytest.mark.parametrize("text,ok", [("cliffs.f:17-346", True), ("cliffs.f:17-347", False),
                                     ("MasterGrid.f:237-268", False), ("errhandle.f:8", True)])
def test_checker_catches_out_of_range(text, ok):
    m = CITE.search(text)
    nums = [int(m.group(2))] + ([int(m.group(3))] if m.group(3) else [])
    assert (max(nums) <= _length(m.group(1))) == ok
