"""Line-by-line numeric diff of two text dumps, with the comparison semantics of
the reference's regression tool (tools/numdiff.py: softEquiv, :70-96; run,
:181-217): columns are split on whitespace; numeric columns must agree within
the relative tolerance (if > 0) and the absolute tolerance (if > 0); other
columns must match exactly when check_text is set; the files must have the
same number of lines.  The reference's regression tests use
`--check-text --absolute 1e-14` (cmake/regression.cmake:19).
"""
from __future__ import annotations

import math
import re
from dataclasses import dataclass, field
from typing import List

_SPLIT = re.compile(r"\s+")


@dataclass
class Report:
    ok: bool = True
    failures: List[str] = field(default_factory=list)
    max_abs_err: float = 0.0

    def fail(self, msg: str) -> None:
        self.ok = False
        if len(self.failures) < 20:
            self.failures.append(msg)


def _split(line: str) -> List[str]:
    parts = _SPLIT.split(line)
    if parts and parts[-1] == "":
        parts.pop()
    if parts and parts[0] == "":
        parts.pop(0)
    return parts


def soft_equiv(ref: float, target: float, rel_tol: float, abs_tol: float) -> bool:
    err = abs(target - ref)
    if rel_tol > 0 and err > abs(ref) * rel_tol:
        return False
    if abs_tol > 0 and err > abs_tol:
        return False
    return True


def compare_lines(expected: List[str], actual: List[str], rel_tol: float = -1.0,
                  abs_tol: float = 1e-14, check_text: bool = True) -> Report:
    rep = Report()
    n = max(len(expected), len(actual))
    for i in range(n):
        e = expected[i].rstrip() if i < len(expected) else ""
        a = actual[i].rstrip() if i < len(actual) else ""
        if e == "" and a != "":
            rep.fail("tested file ended too late")
            break
        if a == "" and e != "":
            rep.fail("tested file ended too early")
            break
        ec, ac = _split(e), _split(a)
        if len(ec) != len(ac):
            rep.fail(f"wrong number of columns in line {i + 1}")
            continue
        for col, (x, y) in enumerate(zip(ec, ac)):
            try:
                xv, yv = float(x), float(y)
            except ValueError:
                if check_text and x != y:
                    rep.fail(f"text did not match in line {i + 1}, column {col}")
                continue
            if math.isnan(xv) or math.isnan(yv):
                if not (math.isnan(xv) and math.isnan(yv)):
                    rep.fail(f"non-equivalence in line {i + 1}, column {col}")
                continue
            rep.max_abs_err = max(rep.max_abs_err, abs(yv - xv))
            if not soft_equiv(xv, yv, rel_tol, abs_tol):
                rep.fail(f"non-equivalence in line {i + 1}, column {col}: {x} vs {y}")
    return rep


def compare_files(expected_path: str, actual_path: str, **kw) -> Report:
    with open(expected_path) as fe, open(actual_path) as fa:
        return compare_lines(fe.read().splitlines(), fa.read().splitlines(), **kw)
