"""Every reference citation in the sources and notes points at lines that exist.

Code and notes cite the reference project as `src/<file>:<line>[-<line>]`
(also `test/...` and bare `<file>.cpp:<line>` in the design tables), so that
a reader can check each restated step against the original.  This test
resolves every such citation against the reference checkout, when it is
mounted, and fails on a missing file or a line range beyond the file's end.
"""
import re
from pathlib import Path

import pytest
from refdir import reference_dir

ROOT = Path(__file__).resolve().parents[1]
REF = reference_dir()

QUALIFIED = re.compile(r"\b((?:src|test|test\.groups)/[\w./-]+\.(?:cpp|h|hpp|txt|R|cva))((?::\d+(?:-\d+)?)"
                       r"(?:,\s*:\d+(?:-\d+)?)*)")
BARE = re.compile(r"(?<![/\w])([A-Za-z_]\w*\.(?:cpp|h|hpp)):(\d+(?:-\d+)?(?:,\s*:?\d+(?:-\d+)?)*)")


def sources():
    for p in ROOT.rglob("*"):
        if not p.is_file() or p.suffix not in {".py", ".cu", ".cuh", ".h", ".cpp", ".c", ".md"}:
            continue
        rel = p.relative_to(ROOT).parts
        if rel[0] in {"_work", "gpurun_out", "baseline"} or p.name in {"SURVEY.md", "BASELINE.md"}:
            continue
        yield p


def line_ranges(text):
    for a, b in re.findall(r"(\d+)(?:-(\d+))?", text):
        yield int(a), int(b) if b else int(a)


def test_reference_citations_resolve():
    if not (REF / "src").is_dir():
        pytest.skip("reference checkout not mounted")
    lines = {}

    def nlines(path):
        if path not in lines:
            lines[path] = len(path.read_text(errors="ignore").splitlines())
        return lines[path]

    bad, checked = [], 0
    for f in sources():
        text = f.read_text(errors="ignore")
        for m in QUALIFIED.finditer(text):
            target = REF / m.group(1)
            checked += 1
            if not target.exists():
                bad.append(f"{f.relative_to(ROOT)}: {m.group(0)} (no such file)")
                continue
            for a, b in line_ranges(m.group(2)):
                if not 1 <= a <= b <= nlines(target):
                    bad.append(f"{f.relative_to(ROOT)}: {m.group(0)} (file has {nlines(target)} lines)")
        for m in BARE.finditer(text):
            target = REF / "src" / m.group(1)
            if not target.exists():
                continue   # a file of this repository
            checked += 1
            for a, b in line_ranges(m.group(2)):
                if not 1 <= a <= b <= nlines(target):
                    bad.append(f"{f.relative_to(ROOT)}: {m.group(0)} (file has {nlines(target)} lines)")
    assert checked > 200
    assert not bad, "\n".join(bad)
