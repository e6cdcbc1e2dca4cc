"""Writes reference_index.json: the line count of every source file of the
UNSFlow2D reference and the line range of every program unit in it
(subroutine, function, program, module; internal ones too).

tests/test_citations.py checks the repository's reference citations
(`CCFVM/main.F90:57-117`, `lusgs.f90:48-124`, ...) against this index, so it
runs without the reference present.  Regenerate with

    python tests/golden/make_reference_index.py /path/to/UNSFlow2D
"""
import json
import re
import sys
from pathlib import Path

START = re.compile(r"^\s*(?:(?:recursive|pure|elemental)\s+)*(?:(?:real|integer|double\s+precision|logical)"
                   r"(?:\s*\([^)]*\))?\s+)?(subroutine|function|program|module)\s+(\w+)", re.I)
END = re.compile(r"^\s*end(?:\s+(?:subroutine|function|program|module)(?:\s+\w+)?)?\s*(?:!.*)?$", re.I)


def units(lines):
    out, stack = [], []
    for i, line in enumerate(lines, 1):
        code = line.split("!", 1)[0]
        if not code.strip():
            continue
        m = START.match(code)
        if m and not re.match(r"^\s*module\s+procedure", code, re.I):
            stack.append([m.group(2), i])
            continue
        if END.match(code) and stack:
            name, a = stack.pop()
            out.append([name, a, i])
    for name, a in stack:  # unterminated (a conflict-marked file): to the end
        out.append([name, a, len(lines)])
    return sorted(out, key=lambda r: r[1])


def main(root: Path) -> None:
    idx = {}
    for f in sorted(root.rglob("*")):
        if not f.is_file() or ".git" in f.parts:
            continue
        rel = f.relative_to(root).as_posix()
        if f.suffix.lower() not in (".f90", ".f", ".inp", "") and f.name != "makefile":
            continue
        lines = f.read_text(errors="replace").splitlines()
        idx[rel] = {"lines": len(lines), "units": units(lines) if f.suffix.lower() in (".f90", ".f") else []}
    out = Path(__file__).with_name("reference_index.json")
    out.write_text(json.dumps(idx, indent=0, sort_keys=True) + "\n")
    print(f"wrote {out} ({len(idx)} files)")


if __name__ == "__main__":
    main(Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference"))
