"""Write tests/golden/reference_calls.json: the Fortran interface the drop-in
module must provide, read from the reference's own sources.

For every SUBROUTINE defined in force.f90 and vverlet.f90 it records the
dummy argument names (file:line), and for every CALL of one of them in
main.f90 and init.f90 the number of actual arguments (file:line).  The shim
test (tests/test_fortran_shim.py) checks tcp_allpair_gb300/fortran/
tcp_gpu_mod.f90 against this file, and against the sources themselves when
they are present.

Usage: python tests/golden/make_reference_calls.py [reference_dir]
"""
from __future__ import annotations

import json
import pathlib
import re
import sys

HERE = pathlib.Path(__file__).resolve().parent
DEFINING = ("force.f90", "vverlet.f90")
CALLING = ("main.f90", "init.f90")


def logical_lines(text: str):
    """(first physical line number, statement) with comments removed and
    '&' continuations joined."""
    out, buf, start = [], "", None
    for no, raw in enumerate(text.splitlines(), 1):
        line, quote = [], None
        for ch in raw:                      # drop '!' comments outside strings
            if quote:
                quote = None if ch == quote else quote
            elif ch in "'\"":
                quote = ch
            elif ch == "!":
                break
            line.append(ch)
        s = "".join(line).strip()
        if not s:
            continue
        if buf and s.startswith("&"):
            s = s[1:].strip()
        if start is None:
            start = no
        if s.endswith("&"):
            buf += s[:-1] + " "
            continue
        out.append((start, buf + s))
        buf, start = "", None
    return out


def split_args(s: str):
    """Top-level comma-separated arguments of the text inside parentheses."""
    args, depth, cur = [], 0, ""
    for ch in s:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == "," and depth == 0:
            args.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        args.append(cur.strip())
    return args


def paren_body(stmt: str, start: int) -> str:
    depth = 0
    for i in range(start, len(stmt)):
        if stmt[i] == "(":
            depth += 1
        elif stmt[i] == ")":
            depth -= 1
            if depth == 0:
                return stmt[start + 1:i]
    raise ValueError(f"unbalanced parentheses: {stmt}")


SUB_RE = re.compile(r"^\s*SUBROUTINE\s+([A-Za-z_]\w*)\s*(\()?", re.I)
CALL_RE = re.compile(r"\bCALL\s+([A-Za-z_]\w*)\s*(\()?", re.I)


def definitions(path: pathlib.Path):
    out = {}
    for no, stmt in logical_lines(path.read_text()):
        m = SUB_RE.match(stmt)
        if not m:
            continue
        args = split_args(paren_body(stmt, m.start(2))) if m.group(2) else []
        out[m.group(1).upper()] = {"name": m.group(1), "file": path.name, "line": no, "args": args}
    return out


def calls(path: pathlib.Path):
    out = []
    for no, stmt in logical_lines(path.read_text()):
        for m in CALL_RE.finditer(stmt):
            nargs = len(split_args(paren_body(stmt, m.start(2)))) if m.group(2) else 0
            out.append({"name": m.group(1).upper(), "file": path.name, "line": no, "nargs": nargs})
    return out


def extract(ref: pathlib.Path):
    defs = {}
    for f in DEFINING:
        defs.update(definitions(ref / f))
    sites = [c for f in CALLING for c in calls(ref / f) if c["name"] in defs]
    return {"defining_files": list(DEFINING), "calling_files": list(CALLING), "definitions": defs,
            "calls": sites}


def main(argv):
    ref = pathlib.Path(argv[1] if len(argv) > 1 else "/root/reference")
    data = extract(ref)
    (HERE / "reference_calls.json").write_text(json.dumps(data, indent=1, sort_keys=True) + "\n")
    print(f"{len(data['definitions'])} definitions, {len(data['calls'])} call sites")


if __name__ == "__main__":
    main(sys.argv)
