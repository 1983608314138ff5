"""runstopping input files (apps/runstopping.C:66-175) as stopping requests.

``load(text)`` reads the JSON runstopping takes on stdin (comments allowed),
checks it like runstopping (same messages) and returns a :class:`StoppingRequest`:
the ion, the target material as a ``LayerSpec`` and the list of energies, built
with the same floating-point accumulation as the reference (a range with "step"
adds, one with "mult" multiplies).  The compiled front-end
``mytrim_gb300/_lib/runstopping_gpu`` (source ``mytrim_gb300/cpp/runstopping_gpu.cpp``)
reads the same files and prints "E S_e" per energy.
"""
import json
from dataclasses import dataclass
from typing import List

from .engine import ElementSpec, LayerSpec
from .runmytrim import InputError, strip_comments, _num


@dataclass
class StoppingRequest:
    Z: int
    m: float
    material: LayerSpec
    energies: List[float]


def load(text: str) -> StoppingRequest:
    try:
        root = json.loads(strip_comments(text))
    except json.JSONDecodeError as e:
        raise InputError(f"cannot parse the input: {e}") from None
    if not isinstance(root, dict) or not isinstance(root.get("stopping"), dict):
        raise InputError("No 'stopping' top level block found in input")
    root = root["stopping"]
    mat = root.get("material")
    if not isinstance(mat, dict):
        raise InputError("Must specify a 'material' block in the input file")
    if not _num(mat.get("rho")):
        raise InputError("Missing 'rho'")
    els = mat.get("elements")
    if not isinstance(els, list):
        raise InputError("Missing 'elements' in material")
    elements = []
    for j, e in enumerate(els):
        for key in ("Z", "mass", "fraction"):
            if not isinstance(e, dict) or not _num(e.get(key)):
                raise InputError(f"Missing '{key}' in element {j}")
        elements.append(ElementSpec(int(e["Z"]), float(e["mass"]), float(e["fraction"])))
    ion = root.get("ion")
    if not isinstance(ion, dict):
        raise InputError("Must specify an 'ion' block in the input file")
    for key in ("Z", "mass"):
        if not _num(ion.get(key)):
            raise InputError(f"Missing '{key}' in ion block")
    en = ion.get("energy")
    energies = []
    if _num(en):
        energies.append(float(en))
    elif isinstance(en, list):
        energies = [float(v) for v in en]
    elif isinstance(en, dict):
        if not _num(en.get("begin")):
            raise InputError("Missing 'begin' in energy block")
        if not _num(en.get("end")):
            raise InputError("Missing 'end' in energy block")
        begin, end = float(en["begin"]), float(en["end"])
        has_step, has_mult = _num(en.get("step")), _num(en.get("mult"))
        if has_step == has_mult:
            raise InputError("Specify either 'step' or 'mult' energy block")
        if has_step:
            step = float(en["step"])
            if not step > 0.0:
                raise InputError("'step' must be positive")
            E = begin
            while E <= end:
                energies.append(E)
                E += step
        else:
            mult = float(en["mult"])
            if mult <= 1.0:
                raise InputError("'mult' must be larger than 1.0")
            E = begin
            while E <= end:
                energies.append(E)
                E *= mult
    else:
        raise InputError("Missing or invalid 'energy' in ion block")
    return StoppingRequest(int(ion["Z"]), float(ion["mass"]), LayerSpec(1.0, float(mat["rho"]), elements), energies)
