"""Every `name.f90:N-M` citation of a reference Fortran source in the code points at lines
that exist: M (and every listed line) is at most the cited file's line count, taken from
tests/golden/reference_line_counts.json (written by make_reference_line_counts.py)."""
import json
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
COUNTS = os.path.join(ROOT, "tests", "golden", "reference_line_counts.json")
SCANNED = ("oracle", "matt_young_mapmaking_gb300", "include", "tests")
SUFFIXES = (".c", ".h", ".cu", ".cpp", ".py", ".f90")
# name.f90 followed by one or more ":a-b,c" groups
CITE = re.compile(r"([A-Za-z_0-9]+\.[fF]90)((?::\d+(?:-\d+)?(?:,\s?\d+(?:-\d+)?)*)+)")


def _sources():
    yield os.path.join(ROOT, "bench.py")
    for top in SCANNED:
        for d, dirs, files in os.walk(os.path.join(ROOT, top)):
            dirs[:] = [x for x in dirs if not x.startswith(("_", "."))]
            for f in files:
                if f.endswith(SUFFIXES):
                    yield os.path.join(d, f)


def test_every_fortran_citation_is_in_range():
    with open(COUNTS) as f:
        counts = json.load(f)
    bad, seen = [], 0
    for path in _sources():
        with open(path, errors="replace") as f:
            for ln, line in enumerate(f, 1):
                for m in CITE.finditer(line):
                    name = m.group(1)
                    assert name in counts, "%s:%d cites unknown file %s" % (path, ln, name)
                    nums = [int(x) for x in re.findall(r"\d+", m.group(2))]
                    seen += 1
                    if max(nums) > counts[name]["lines"] or min(nums) < 1:
                        bad.append("%s:%d %s%s (file has %d lines)"
                                   % (os.path.relpath(path, ROOT), ln, name, m.group(2),
                                      counts[name]["lines"]))
    assert seen > 50, "citation scan found only %d citations" % seen
    assert not bad, "citations past the end of the cited file:\n" + "\n".join(bad)
