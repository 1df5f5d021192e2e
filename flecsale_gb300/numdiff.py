"""Line-by-line numeric diff of two text dumps, with the comparison semantics of
the reference's regression tool (tools/numdiff.py: softEquiv, :70-96; run,
:181-217): columns are split on commas, semicolons and whitespace (:23);
numeric columns must agree within the relative tolerance (if > 0) and the
absolute tolerance (if > 0); other columns must match exactly when check_text
is set; the comparison ends at the first empty line of the expected file, and
the tested file must end there too.  The reference's regression tests use
`--check-text --absolute 1e-14` (cmake/regression.cmake:19).

Command line, with the reference tool's options and exit status (:222-266):
    python -m flecsale_gb300.numdiff [-c] [-a ABS] [-r REL] [-t TOL] [-q] [-v] expected actual
"""
from __future__ import annotations

import argparse
import math
import re
import sys
from dataclasses import dataclass, field
from typing import List, Optional

_SPLIT = re.compile(r",|\s+|;")


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
        if e == "":
            if a != "":
                rep.fail("tested file ended too late")
            break
        if a == "":
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


def main(argv: Optional[List[str]] = None) -> int:
    """The reference tool's command line: exit status 0 and SUCCESS when the
    files agree, 1 and FAILURE (after one ">>>> reason" line per failure, at
    most 20) otherwise.  Without -r and -a both tolerances are -t (1e-15)."""
    ap = argparse.ArgumentParser(description="numeric diff of two text files")
    ap.add_argument("-q", "--quiet", action="store_true")
    ap.add_argument("-v", "--verbose", action="count", default=0)
    ap.add_argument("-c", "--check-text", action="store_true")
    ap.add_argument("-t", "--tolerance", type=float, default=1e-15)
    ap.add_argument("-r", "--relative", type=float, default=-1.0)
    ap.add_argument("-a", "--absolute", type=float, default=-1.0)
    ap.add_argument("files", nargs="*")
    args = ap.parse_args(argv)
    if len(args.files) != 2:
        ap.print_help()
        return 1
    rel, abs_ = args.relative, args.absolute
    if rel < 0 and abs_ < 0:
        rel = abs_ = args.tolerance
    rep = compare_files(args.files[0], args.files[1], rel_tol=rel, abs_tol=abs_,
                        check_text=args.check_text)
    for msg in rep.failures:
        print(">>>> " + msg)
    print("SUCCESS" if rep.ok else "FAILURE")
    return 0 if rep.ok else 1


if __name__ == "__main__":
    sys.exit(main())
