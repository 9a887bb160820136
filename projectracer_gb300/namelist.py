"""Reader for the reference's Fortran namelist file (inputs.nml).

The reference reads four groups with ``read(nml=...)`` (main.f90:11-21; groups declared at
basics.f90:54-66).  This reader understands the subset of namelist syntax that file uses:
``key=value`` pairs, ``!`` comments, array elements such as ``RaC(1)=0.5d5``, and Fortran real
literals with ``d`` exponents.  A ``&gpu`` group (precision, guess mode) is accepted alongside,
so a reference-compatible inputs.nml stays valid.
"""

from __future__ import annotations

import re

_ASSIGN = re.compile(r"^\s*([A-Za-z_][A-Za-z0-9_]*)\s*(\(\s*(\d+)\s*\))?\s*=\s*(.*)$")


def _value(text: str):
    text = text.strip().rstrip(",").strip()
    low = text.lower()
    if low in (".true.", "t", ".t."):
        return True
    if low in (".false.", "f", ".f."):
        return False
    if text.startswith(("'", '"')):
        return text.strip("'\"")
    num = low.replace("d", "e")
    try:
        if re.fullmatch(r"[+-]?\d+", num):
            return int(num)
        return float(num)
    except ValueError:
        return text


def parse_namelist(text: str) -> dict[str, dict[str, object]]:
    """Return {group: {key: value}}; array elements become key(1) etc. -> key with index 1."""
    groups: dict[str, dict[str, object]] = {}
    current = None
    for raw in text.splitlines():
        line = raw.split("!", 1)[0].rstrip()
        if not line.strip():
            continue
        stripped = line.strip()
        if stripped.startswith("&"):
            current = stripped[1:].split()[0].lower()
            groups.setdefault(current, {})
            continue
        if stripped == "/":
            current = None
            continue
        if current is None:
            continue
        m = _ASSIGN.match(line)
        if not m:
            continue
        key = m.group(1).lower()
        if m.group(3) is not None:
            key = f"{key}({int(m.group(3))})"
        groups[current][key] = _value(m.group(4))
    return groups


def read_namelist(path: str) -> dict[str, dict[str, object]]:
    with open(path, "r", encoding="utf-8") as fh:
        return parse_namelist(fh.read())
