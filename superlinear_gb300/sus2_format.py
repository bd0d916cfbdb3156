"""Text I/O for the native ``.sus2`` SUS2-SH model format (host side).

The format is the reference's: an ``MTP`` header, ``key = value`` lines whose
values may be brace lists spanning several lines, and a ``radial_coeffs`` block
(a ``0-0`` sub-header followed by one ``{...}`` row per radial function).
Reader semantics follow ``interfaces/lammps/ML-SUS2/sus2_sl_model.cpp:174-257``
(``Model::load``).  The CUDA library parses the file itself in C++; this module
is used by the workload generators and tests to read, rewrite and emit models.
"""
from __future__ import annotations

import re
from collections import OrderedDict

__all__ = ["read_sus2", "write_sus2", "parse_list", "format_list"]


def parse_list(text: str) -> list:
    """Flatten a brace list such as ``{{1, 2}, {3}}`` into ``[1.0, 2.0, 3.0]``."""
    body = text.replace("{", " ").replace("}", " ").replace(",", " ")
    return [float(tok) for tok in body.split()]


def format_list(values, nested: int | None = None) -> str:
    """Format numbers as a brace list; ``nested=w`` groups rows of width ``w``."""
    def fmt(v):
        v = float(v)
        return str(int(v)) if v.is_integer() and abs(v) < 1e15 and nested is not None else f"{v:.17e}"
    vals = [fmt(v) for v in values]
    if nested:
        rows = ["{" + ", ".join(vals[i:i + nested]) + "}" for i in range(0, len(vals), nested)]
        return "{" + ", ".join(rows) + "}"
    return "{" + ", ".join(vals) + "}"


def read_sus2(path: str) -> "OrderedDict[str, str]":
    """Return the ordered ``key -> raw value text`` map of a ``.sus2`` file.

    The radial block is returned under ``radial_coeffs`` as one flat brace list
    (rows concatenated), matching ``sus2_sl_model.cpp:189-197``.
    """
    fields: "OrderedDict[str, str]" = OrderedDict()
    radial_rows: list[str] = []
    in_radial = False
    header = False
    with open(path) as fh:
        lines = iter(fh.read().splitlines())
    for raw in lines:
        line = raw.strip()
        if not line or line.startswith("#"):
            continue
        if not header:
            if line != "MTP":
                raise ValueError("missing MTP header")
            header = True
            continue
        if "=" not in line:
            if line == "radial_coeffs":
                in_radial = True
                fields["radial_coeffs"] = ""  # keeps the block's position in the file
                continue
            if not in_radial:
                raise ValueError(f"unrecognized line: {line}")
            if line == "0-0":
                continue
            radial_rows.append(line)
            continue
        in_radial = False
        key, value = (s.strip() for s in line.split("=", 1))
        depth = value.count("{") - value.count("}")
        while depth > 0:
            nxt = next(lines).strip()
            value += " " + nxt
            depth += nxt.count("{") - nxt.count("}")
        if key in fields:
            raise ValueError(f"duplicate field {key}")
        fields[key] = value
    if radial_rows:
        fields["radial_coeffs"] = "{" + ", ".join(radial_rows) + "}"
    elif "radial_coeffs" in fields:
        del fields["radial_coeffs"]
    return fields


# Keys written indented under radial_basis_type, as the reference writer does.
_RADIAL_META = ("scaling_inner", "min_dist", "max_dist", "angular_max_dist", "radial_basis_size",
                "radial_cutoff_type", "radial_cutoff_p", "radial_funcs_count")


def write_sus2(path: str, fields: "OrderedDict[str, str]") -> None:
    """Write ``fields`` back as a ``.sus2`` file the reference loaders accept.

    ``radial_coeffs`` (flat list of F rows of width B+C) is emitted as the
    indented block at its recorded position, or else right after
    ``scal_coeffs`` -- the order the trainer's sequential reader expects
    (``dev_src/mtpr.cpp:5100-5150``).
    """
    out = ["MTP"]
    radial = fields.get("radial_coeffs")
    B = int(float(fields["radial_basis_size"])) if "radial_basis_size" in fields else 0
    C = int(float(fields["species_count"])) if "species_count" in fields else 0
    keys = list(fields.keys())
    if radial is not None and keys.index("radial_coeffs") < keys.index("scal_coeffs"):
        keys.remove("radial_coeffs")
        keys.insert(keys.index("scal_coeffs") + 1, "radial_coeffs")

    def emit_radial():
        vals = parse_list(radial)
        w = B + C
        out.append("\tradial_coeffs")
        out.append("\t\t0-0")
        for r in range(len(vals) // w):
            out.append("\t\t\t" + format_list(vals[r * w:(r + 1) * w]))

    for key in keys:
        if key == "radial_coeffs":
            emit_radial()
            continue
        indent = "\t" if key in _RADIAL_META else ""
        out.append(f"{indent}{key} = {fields[key]}")
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")


def as_int(fields, key, default=None):
    if key not in fields:
        return default
    return int(float(fields[key]))


_TOKEN = re.compile(r"\s+")
