"""Reader for MuMFiM's microscale job files (the ``fiber_only.yaml`` format).

The reference loads these with yaml-cpp into ``MicroCase`` records
(src/mumfim/microscale/MicroFOParams.cc:184-330): a sequence of cases, each
with ``Case`` (name), ``Problem Definition`` (``Mesh``, ``Deformation
Gradient``), ``Solution Strategy`` and ``Output``. PyYAML is not available
here, so this module reads the subset of YAML those files use: block
mappings and sequences by indentation, flow sequences (``[a, [b, c]]``),
``#`` comments, and plain or quoted scalars (numbers, ``true``/``false``,
strings).
"""
from __future__ import annotations

import os
import re
from dataclasses import dataclass, field
from typing import Any, Dict, List

from .strategy import SolutionStrategy


class JobFileError(ValueError):
    pass


_NUM = re.compile(r"^[+-]?(\d+\.?\d*|\.\d+)([eE][+-]?\d+)?$")


def _strip_comment(line: str) -> str:
    out, quote = [], None
    for ch in line:
        if quote:
            if ch == quote:
                quote = None
        elif ch in "\"'":
            quote = ch
        elif ch == "#":
            break
        out.append(ch)
    return "".join(out).rstrip()


def _scalar(tok: str) -> Any:
    tok = tok.strip()
    if len(tok) >= 2 and tok[0] == tok[-1] and tok[0] in "\"'":
        return tok[1:-1]
    low = tok.lower()
    if low in ("true", "yes", "on"):
        return True
    if low in ("false", "no", "off"):
        return False
    if low in ("null", "~", ""):
        return None
    if _NUM.match(tok):
        return float(tok) if any(c in tok for c in ".eE") else int(tok)
    return tok


def _flow(text: str) -> Any:
    """A flow sequence such as [1, 0, [1, 0, 0]]."""
    pos = 0

    def item():
        nonlocal pos
        while pos < len(text) and text[pos] == " ":
            pos += 1
        if pos < len(text) and text[pos] == "[":
            pos += 1
            seq = []
            while True:
                while pos < len(text) and text[pos] == " ":
                    pos += 1
                if pos < len(text) and text[pos] == "]":
                    pos += 1
                    return seq
                seq.append(item())
                while pos < len(text) and text[pos] == " ":
                    pos += 1
                if pos < len(text) and text[pos] == ",":
                    pos += 1
                elif pos < len(text) and text[pos] == "]":
                    continue
                else:
                    raise JobFileError(f"bad flow sequence: {text!r}")
        start = pos
        while pos < len(text) and text[pos] not in ",]":
            pos += 1
        return _scalar(text[start:pos])

    val = item()
    if text[pos:].strip():
        raise JobFileError(f"trailing text in {text!r}")
    return val


def _value(tok: str) -> Any:
    tok = tok.strip()
    return _flow(tok) if tok.startswith("[") else _scalar(tok)


def parse_yaml_subset(text: str) -> Any:
    lines = []
    for raw in text.splitlines():
        line = _strip_comment(raw)
        if line.strip():
            if "\t" in line[: len(line) - len(line.lstrip())]:
                raise JobFileError("tabs in indentation")
            lines.append((len(line) - len(line.lstrip(" ")), line.strip()))
    pos = 0

    def block(indent: int) -> Any:
        nonlocal pos
        if pos >= len(lines):
            return None
        if lines[pos][1].startswith("- ") or lines[pos][1] == "-":
            seq = []
            while pos < len(lines) and lines[pos][0] == indent and (
                    lines[pos][1].startswith("- ") or lines[pos][1] == "-"):
                rest = lines[pos][1][1:].lstrip()
                if not rest:
                    pos += 1
                    seq.append(block(lines[pos][0]) if pos < len(lines) and lines[pos][0] > indent
                               else None)
                    continue
                # "- key: value" opens a mapping at the item's content column
                lines[pos] = (indent + len(lines[pos][1]) - len(rest), rest)
                seq.append(block(lines[pos][0]))
            return seq
        mapping: Dict[str, Any] = {}
        while pos < len(lines) and lines[pos][0] == indent:
            text_ = lines[pos][1]
            if text_.startswith("- "):
                raise JobFileError(f"unexpected sequence item: {text_!r}")
            key, sep, rest = text_.partition(":")
            if not sep:
                raise JobFileError(f"expected 'key: value', got {text_!r}")
            pos += 1
            if rest.strip():
                mapping[key.strip()] = _value(rest)
            elif pos < len(lines) and lines[pos][0] > indent:
                mapping[key.strip()] = block(lines[pos][0])
            elif pos < len(lines) and lines[pos][0] == indent and lines[pos][1].startswith("- "):
                mapping[key.strip()] = block(indent)
            else:
                mapping[key.strip()] = None
        if pos < len(lines) and lines[pos][0] > indent:
            raise JobFileError(f"bad indentation at {lines[pos][1]!r}")
        return mapping

    doc = block(lines[0][0]) if lines else None
    if pos != len(lines):
        raise JobFileError(f"could not read from {lines[pos][1]!r}")
    return doc


@dataclass
class MicroCase:
    """One case of a job file (MicroFOParams.h: MicroCase)."""

    name: str
    mesh: str
    F: List[float]
    solution: Dict[str, Any] = field(default_factory=dict)
    output: Dict[str, Any] = field(default_factory=dict)

    def strategy(self) -> SolutionStrategy:
        """The explicit strategy the batched analysis takes from this case:
        the damping; the batched kernels fix the critical-step factor at 0.8
        and relax to a residual of 1e-6
        (BatchedFiberRVEAnalysisExplicitTeamOuterLoop.h:312,371)."""
        return SolutionStrategy(visc_damp_coeff=float(self.solution["Viscous Damping Factor"]),
                                crit_time_scale_factor=0.8, residual_tol=1e-6)

    @property
    def orientation_2d_axis(self):
        v = self.output.get("2D Orientation Tensor")
        if isinstance(v, list) and len(v) == 2 and v[0] and isinstance(v[1], list):
            return [float(x) for x in v[1]]
        return None


def _case(node: Any) -> MicroCase:
    if not isinstance(node, dict):
        raise JobFileError("a case must be a mapping")
    try:
        pd = node["Problem Definition"]
        ss = node["Solution Strategy"]
        F = pd["Deformation Gradient"]
        mesh = pd["Mesh"]
    except (KeyError, TypeError) as e:
        raise JobFileError(f"missing field {e}") from None
    if not isinstance(F, list) or len(F) != 9:
        raise JobFileError("Deformation Gradient must have 9 entries")
    if not isinstance(ss, dict) or ss.get("Solver Type") != "Explicit":
        raise JobFileError("the batched analysis needs 'Solver Type: Explicit'")
    if "Viscous Damping Factor" not in ss:
        raise JobFileError("missing 'Viscous Damping Factor'")
    return MicroCase(str(node.get("Case", "")), str(mesh), [float(x) for x in F], ss,
                     node.get("Output") or {})


def load_micro_cases(path: str) -> List[MicroCase]:
    """All cases of a job file (loadMicroFOFromYamlFile, MicroFOParams.cc:330-340)."""
    with open(path) as fh:
        doc = parse_yaml_subset(fh.read())
    if not isinstance(doc, list) or not doc:
        raise JobFileError("a job file is a sequence of cases")
    return [_case(c) for c in doc]


def resolve_mesh(case: MicroCase, job_path: str) -> str:
    """The network file of a case: as given (relative to the working
    directory, as the reference opens it), else next to the job file."""
    if os.path.exists(case.mesh):
        return case.mesh
    alt = os.path.join(os.path.dirname(os.path.abspath(job_path)), case.mesh)
    return alt if os.path.exists(alt) else case.mesh
