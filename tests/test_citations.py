"""Reference citations in the repository point at real lines.

Every `CCFVM/...`, `NCFVM/...` or `MeshGen/...` citation with line numbers,
and every bare `name.F90:N-M` / `name.f90:N-M` citation, in a tracked text
file must name lines that exist in the reference file it cites.  Where the
text just before a citation names a program unit of that file
("save_old (CCFVM/solution.F90:118-132)"), the cited lines must overlap that
unit.  The line counts and unit ranges come from
tests/golden/reference_index.json (make_reference_index.py), so the test
needs no copy of the reference.
"""
import json
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
INDEX = json.loads((ROOT / "tests" / "golden" / "reference_index.json").read_text())
CODE = (".py", ".cu", ".cuh", ".cpp", ".hpp", ".h", ".inc")
# Documents are checked when they carry this marker: the repository's own
# documentation does; documents written about the repository by others cite
# the reference in their own way and are not part of the product.
MARK = "<!-- reference citations in this file are checked by tests/test_citations.py -->"

FULL = re.compile(r"((?:CCFVM|NCFVM|MeshGen)/[A-Za-z0-9_/.]+?\.(?:[fF]90|f|inp)|(?:CCFVM|NCFVM|MeshGen)/makefile)"
                  r":(\d+(?:-\d+)?(?:,\s?\d+(?:-\d+)?)*)")
BARE = re.compile(r"(?<![/\w.])([A-Za-z_][A-Za-z0-9_]*\.[fF]90):(\d+(?:-\d+)?(?:,\s?\d+(?:-\d+)?)*)")
BY_NAME: dict[str, list[str]] = {}
for _rel in INDEX:
    BY_NAME.setdefault(_rel.rsplit("/", 1)[-1], []).append(_rel)


def _ranges(spec: str):
    for part in spec.replace(" ", "").split(","):
        a, _, b = part.partition("-")
        yield int(a), int(b) if b else int(a)


NOT_SOURCE = {"_work", "gpurun_out", "_build", "lib", "baseline", "build", "__pycache__", ".git", ".pytest_cache"}


def _tracked():
    """The repository's text files: git's list where there is a checkout, else
    a walk of the tree without build, scratch and output folders."""
    out = subprocess.run(["git", "ls-files"], cwd=ROOT, capture_output=True, text=True)
    if out.returncode == 0 and out.stdout.strip():
        files = out.stdout.split()
    else:
        files = [str(f.relative_to(ROOT)) for f in ROOT.rglob("*")
                 if f.is_file() and not (set(f.relative_to(ROOT).parts[:-1]) & NOT_SOURCE)]
    def checked(f):
        if f.startswith("_work/"):
            return False
        if f.endswith(CODE):
            return True
        return f.endswith(".md") and MARK in (ROOT / f).read_text(errors="replace")
    return sorted(f for f in files if checked(f))


def _citations():
    for fn in _tracked():
        text = (ROOT / fn).read_text(errors="replace")
        for ln, line in enumerate(text.splitlines(), 1):
            prev = 0
            found = [(m.start(), m.end(), m.group(1), m.group(2)) for m in FULL.finditer(line)]
            spans = [(s, e) for s, e, _, _ in found]
            for m in BARE.finditer(line):
                if any(s <= m.start() < e for s, e in spans):
                    continue
                cands = BY_NAME.get(m.group(1), [])
                rel = cands[0] if len(cands) == 1 else None
                found.append((m.start(), m.end(), rel or m.group(1), m.group(2)))
            for s, e, rel, spec in sorted(found):
                yield fn, ln, line[prev:s], rel, spec
                prev = e


CITES = list(_citations())


def test_the_documentation_is_checked():
    docs = [f for f in _tracked() if f.endswith(".md")]
    assert len(docs) >= 3 and any("/" not in f for f in docs), docs
    assert any(c[0].endswith(".md") for c in CITES)


def test_some_citations_found():
    assert len(CITES) > 100


@pytest.mark.parametrize("fn,ln,before,rel,spec", CITES, ids=[f"{c[0]}:{c[1]}:{c[3]}:{c[4]}" for c in CITES])
def test_citation_in_range_and_on_the_named_unit(fn, ln, before, rel, spec):
    assert rel in INDEX, f"{fn}:{ln}: {rel} is not a reference file"
    info = INDEX[rel]
    rngs = list(_ranges(spec))
    for a, b in rngs:
        assert 1 <= a <= b <= info["lines"], f"{fn}:{ln}: {rel}:{spec} outside the file's {info['lines']} lines"
    # the program unit named closest before the citation, if any
    names = {u[0].lower(): (u[1], u[2]) for u in info["units"]}
    words = re.findall(r"[A-Za-z_][A-Za-z0-9_]*", before)
    named = next((w.lower() for w in reversed(words) if w.lower() in names), None)
    if named is not None:
        ua, ub = names[named]
        assert any(not (b < ua or a > ub) for a, b in rngs), \
            f"{fn}:{ln}: {named} is {rel}:{ua}-{ub}, the citation says {spec}"
