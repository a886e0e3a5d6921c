"""Every citation of the reference (`name.jl:N` or `name.jl:N-M`) in this repository's files
points at lines that exist in the cited file of the reference source tree.

A bare file name resolves to the reference file of that name; where several share it (such as
`window.jl` in `src/fbp/` and `test/fbp/`), to the one under `src/` (or `ext/`); a citation of a
test file names its directory (`test/fbp/window.jl:9-15`).  The reference tree is read from
$SGB_REFERENCE (default /root/reference); without it the test is skipped."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("SGB_REFERENCE", "/root/reference")
# files written by the build's driver, not by this project
FOREIGN = ("SURVEY.md", "VERDICT.md", "ADVICE.md", "BASELINE.md", "BASELINE.json")
CITE = re.compile(r"((?:[\w.-]+/)*[\w.-]+\.jl):(\d+)(?:-(\d+))?")


def _reference_files():
    out = {}
    for dp, _, fn in os.walk(REF):
        for f in fn:
            if f.endswith(".jl"):
                p = os.path.join(dp, f)
                with open(p, errors="replace") as fh:
                    out[os.path.relpath(p, REF)] = sum(1 for _ in fh)
    return out


def _resolve(name, files):
    cands = [p for p in files if p == name or p.endswith("/" + name)]
    if len(cands) == 1:
        return cands[0]
    src = [p for p in cands if p.startswith(("src/", "ext/"))]
    return src[0] if len(src) == 1 else None


def _repo_files():
    try:
        r = subprocess.run(["git", "ls-files"], cwd=ROOT, capture_output=True, text=True, check=True)
        files = r.stdout.split()
    except Exception:
        files = []
        for dp, dn, fn in os.walk(ROOT):
            dn[:] = [d for d in dn if d not in (".git", "_work", "gpurun_out", "baseline", "_build", "__pycache__")]
            files += [os.path.relpath(os.path.join(dp, f), ROOT) for f in fn]
    keep = []
    for f in files:
        base = os.path.basename(f)
        if base in FOREIGN or base.startswith(("BENCH_", "GPUTEST_", "SCALE_", "MULTICHIP_")):
            continue
        if f.endswith((".npz", ".so", ".o", ".png")):
            continue
        keep.append(f)
    return keep


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")), reason="reference source tree not mounted")
def test_reference_citations_exist():
    files = _reference_files()
    bad, n = [], 0
    for f in _repo_files():
        path = os.path.join(ROOT, f)
        if not os.path.isfile(path):
            continue
        with open(path, errors="replace") as fh:
            for ln, line in enumerate(fh, 1):
                for m in CITE.finditer(line):
                    n += 1
                    a = int(m.group(2))
                    b = int(m.group(3) or a)
                    r = _resolve(m.group(1), files)
                    if r is None:
                        bad.append(f"{f}:{ln}: {m.group(0)} names no unique reference file")
                    elif not 1 <= a <= b <= files[r]:
                        bad.append(f"{f}:{ln}: {m.group(0)} is outside {r} ({files[r]} lines)")
    assert n > 100, f"only {n} citations found"
    assert not bad, "\n".join(bad)
