"""runmytrim input files (apps/runmytrim.C:103-285) as engine simulations.

``load(text)`` reads the JSON that runmytrim takes on stdin -- including the
``//`` and ``/* */`` comments jsoncpp accepts -- checks it the way runmytrim
does (same messages) and returns a :class:`RunmytrimInput`: the ``SimSpec`` of
the run plus the output settings.  The compiled front-end
``mytrim_gb300/_lib/runmytrim_gpu`` (source ``mytrim_gb300/cpp/runmytrim_gpu.cpp``)
reads the same files and writes runmytrim's output files.

Semantics kept from runmytrim: the sample is a ``SampleLayers`` of the summed
thickness x 100 x 100 with periodic boundaries (sample.C:31), primaries start
at (0, 50, 50) moving along +x (runmytrim.C:293-298), elements default to
Edisp 25 and Elbind 3 eV (element.C:25), the ion's final energy defaults to
3 eV (ion.C:26), and the output type selects the plugin: ``vaccount`` and
``vacenergycount`` follow every recoil unless ``primaries_only`` is set,
``range`` follows generation 0 only and counts Kinchin-Pease vacancies
(apps/include/TrimRange.h:16).  ``options.threads`` is accepted and ignored.
"""
import json
from dataclasses import dataclass
from typing import Optional

from . import _ffi as F
from .engine import ElementSpec, LayerSpec, SimSpec

OUTPUT_TYPES = ("vaccount", "vacenergycount", "range")
OUTPUT_SUFFIX = {"vaccount": "_vac.dat", "vacenergycount": "_evac.dat", "range": "_ranges.dat"}


class InputError(ValueError):
    """An input runmytrim would reject (the message is runmytrim's)."""


@dataclass
class RunmytrimInput:
    sim: SimSpec
    output_type: str
    base: str
    seed: Optional[int]          # None: runmytrim would draw one from /dev/random
    scale: float = 1.0
    threads: int = 1

    @property
    def output_file(self) -> str:
        return self.base + OUTPUT_SUFFIX[self.output_type]


def strip_comments(text: str) -> str:
    """Remove // line comments, /* */ block comments and trailing commas (before a
    closing } or ]) outside strings: the jsoncpp syntax runmytrim accepts."""
    out = []
    i, n = 0, len(text)
    in_str = False
    while i < n:
        c = text[i]
        if in_str:
            out.append(c)
            if c == "\\" and i + 1 < n:
                out.append(text[i + 1])
                i += 2
                continue
            if c == '"':
                in_str = False
            i += 1
        elif c == '"':
            in_str = True
            out.append(c)
            i += 1
        elif text.startswith("//", i):
            j = text.find("\n", i)
            i = n if j < 0 else j
        elif text.startswith("/*", i):
            j = text.find("*/", i + 2)
            i = n if j < 0 else j + 2
        elif c in "}]":
            # drop a trailing comma (and the whitespace after it) before the bracket
            k = len(out) - 1
            while k >= 0 and out[k] in " \t\r\n":
                k -= 1
            if k >= 0 and out[k] == ",":
                del out[k:]
            out.append(c)
            i += 1
        else:
            out.append(c)
            i += 1
    return "".join(out)


def _num(v) -> bool:
    return isinstance(v, (int, float)) and not isinstance(v, bool)


def load(text: str) -> RunmytrimInput:
    try:
        root = json.loads(strip_comments(text))
    except json.JSONDecodeError as e:
        raise InputError(f"cannot parse the input: {e}") from None
    if not isinstance(root, dict) or not isinstance(root.get("mytrim"), dict):
        raise InputError("No 'mytrim' top level block found in input")
    root = root["mytrim"]
    opts = root.get("options") if isinstance(root.get("options"), dict) else {}
    threads = int(opts["threads"]) if _num(opts.get("threads")) else 1
    seed = int(opts["seed"]) if _num(opts.get("seed")) else None
    scale = float(opts["scale"]) if _num(opts.get("scale")) else 1.0

    sample = root.get("sample")
    if not isinstance(sample, dict):
        raise InputError("Must specify a 'sample' block in the input file")
    jl = sample.get("layers")
    if not isinstance(jl, list):
        raise InputError("sample.layers must be an array")
    for i, l in enumerate(jl):
        if not isinstance(l, dict) or not _num(l.get("thickness")):
            raise InputError(f"No 'thickness' found for layer {i}")

    out = root.get("output")
    if not isinstance(out, dict):
        raise InputError("Must specify an 'output' block in the input file")
    if not isinstance(out.get("type"), str):
        raise InputError("output.type must be a string")
    otype = out["type"]
    if otype not in OUTPUT_TYPES:
        raise InputError(f"Unknown output type {otype}")
    base = out["base"] if isinstance(out.get("base"), str) else ""
    primaries_only = bool(out["primaries_only"]) if isinstance(out.get("primaries_only"), bool) else False

    layers = []
    # runmytrim fills one Element object for all layers: an omitted edisp / elbind
    # keeps the value of the element before it (runmytrim.C:208-251; for its
    # first thread, whose sample this is)
    edisp, elbind = 25.0, 3.0
    for i, l in enumerate(jl):
        if not _num(l.get("rho")):
            raise InputError(f"Missing 'rho' in layer {i}")
        je = l.get("elements")
        if not isinstance(je, list):
            raise InputError(f"Missing 'elements' in layer {i}")
        els = []
        for j, e in enumerate(je):
            for key in ("Z", "mass", "fraction"):
                if not isinstance(e, dict) or not _num(e.get(key)):
                    raise InputError(f"Missing '{key}' in element {j} in layer {i}")
            if _num(e.get("edisp")):
                edisp = float(e["edisp"])
            if _num(e.get("elbind")):
                elbind = float(e["elbind"])
            els.append(ElementSpec(int(e["Z"]), float(e["mass"]), float(e["fraction"]), edisp, elbind))
        layers.append(LayerSpec(float(l["thickness"]), float(l["rho"]), els))

    ion = root.get("ion")
    if not isinstance(ion, dict):
        raise InputError("Must specify an 'ion' block in the input file")
    for key in ("Z", "mass", "energy", "number"):
        if not _num(ion.get(key)):
            raise InputError(f"Missing '{key}' in ion block")
    Ef = float(ion["final_energy"]) if _num(ion.get("final_energy")) else 3.0

    sim = SimSpec(layers=layers, Z=int(ion["Z"]), m=float(ion["mass"]), E=float(ion["energy"]),
                  n_primaries=int(ion["number"]), Ef=Ef, bc=(F.BC_PBC, F.BC_PBC, F.BC_PBC),
                  mode="range" if otype == "range" else "vaccount", primaries_only=primaries_only)
    return RunmytrimInput(sim=sim, output_type=otype, base=base, seed=seed, scale=scale, threads=threads)
