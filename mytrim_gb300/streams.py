"""Text streams of the reference's event-logging TrimBase subclasses, written from
the engine's event log (``Engine.set_event_log`` / ``Engine.events``).

* ``defect_log`` -- TrimDefectLog (trim.C:467-483): "V <ion>" for every vacancy
  (the displaced recoil), "I", "S" or "R" <ion> for every member that came to rest
  as an interstitial, substitutional or replacement;
* ``vac_map`` -- TrimVacMap (trim.C:484-501): the vacancy map of up to three target
  species over the sample's (x, y) extent;
* ``history`` -- TrimHistory (trim.h:139-153): the moving atom's positions at its
  displaced recoils;
* ``md_tag_log`` -- IonMDTag's stream form (ion.C:98-104) of the members at rest:
  "<ion> <_md>";
* ``phonon_log`` -- TrimPhononOut (trim.C:504-527): "<E> <ion>" for every energy
  left in the lattice: the binding energy of each displaced recoil, the energy plus
  binding energy of each recoil below the displacement energy, the residual energy
  of each member that came to rest.

``<ion>`` is IonBase's stream form (ion.C:74-79): x y z Z m E id gen tag, numbers as
std::ostream prints them (six significant digits).  The engine has no sequential
ion ids: the member's path key stands in for the id (of the member that raised the
event).  The tag is IonBase::_tag: the index of the cluster a followed recoil was
created in (sampleClusters), else -1.  The GPU writes events in no particular
order; the lines are sorted by simulation, primary, path key, kind and position.
"""
from typing import Iterable, TextIO

import numpy as np

from . import _ffi as F

_REST_LETTER = {1: "R", 2: "S", 3: "I"}  # IonBase::StateType (ion.h:75-84)


def _g(v: float) -> str:
    return "%g" % v


def _ion(e) -> str:
    return (f"{_g(e['x'])} {_g(e['y'])} {_g(e['z'])} {int(e['Z'])} {_g(e['m'])} {_g(e['E'])} "
            f"{int(e['key'])} {int(e['gen'])} {int(e['tag'])} ")


def _sorted(events: np.ndarray) -> np.ndarray:
    """by simulation, primary, path key of the member that raised the event, kind,
    then position (one member's events of one kind lie a flight path apart)"""
    order = np.lexsort((events["z"], events["y"], events["x"], events["kind"], events["key"], events["primary"],
                        events["sim"]))
    return events[order]


def defect_log(events: np.ndarray) -> Iterable[str]:
    """Lines of TrimDefectLog for events logged with kinds EV_VACANCY and EV_REST."""
    for e in _sorted(events):
        k = int(e["kind"])
        if k == F.EV_VACANCY:
            yield "V " + _ion(e)
        elif k == F.EV_REST and int(e["state"]) in _REST_LETTER:
            yield _REST_LETTER[int(e["state"])] + " " + _ion(e)


def phonon_log(events: np.ndarray) -> Iterable[str]:
    """Lines of TrimPhononOut for events logged with kinds EV_BRANCH, EV_DISSIPATE
    and EV_REST."""
    for e in _sorted(events):
        k = int(e["kind"])
        if k == F.EV_BRANCH:
            yield f"{_g(e['aux'])} " + _ion(e)
        elif k == F.EV_DISSIPATE:
            yield f"{_g(e['E'] + e['aux'])} " + _ion(e)
        elif k == F.EV_REST:
            yield f"{_g(e['E'])} " + _ion(e)


def md_tag_log(events: np.ndarray) -> Iterable[str]:
    """IonMDTag's stream form (ion.C:98-104: the IonBase fields, then _md) of every
    member that came to rest (events logged with kind EV_REST; SimSpec.md_tag_Z sets
    the MD-gap rule), as the demo programs print their tagged ions."""
    for e in _sorted(events):
        if int(e["kind"]) == F.EV_REST:
            yield _ion(e) + f"{int(e['md'])} "


def vac_map(events: np.ndarray, w, z, mx: int = 20, my: int = 20) -> np.ndarray:
    """TrimVacMap (trim.C:484-501) from events logged with kind EV_VACANCY: counts of
    vacancies left by atoms of Z = z[0], z[1] (and z[2]) on an mx x my map of the
    displaced recoil's (x, y) over the sample's extent w[0] x w[1], indices
    int(x mx / w0) reduced modulo mx as the reference does (x -= int(x / mx) mx).
    Returns an (mx, my, 3) integer array.  Positions below zero give negative
    indices, which the reference writes out of its array's bounds; they are not
    counted here."""
    out = np.zeros((mx, my, 3), dtype=np.int64)
    zs = list(z) + [-1] * (3 - len(z))
    for e in events[events["kind"] == F.EV_VACANCY]:
        x = int(e["x"] * mx / w[0])
        y = int(e["y"] * my / w[1])
        x -= int(x / mx) * mx
        y -= int(y / my) * my
        if x < 0 or y < 0:
            continue
        Z = int(e["Z"])
        for k in range(3):
            if Z == zs[k]:
                out[x, y, k] += 1
                break
    return out


def history(events: np.ndarray) -> np.ndarray:
    """TrimHistory::getHistory (trim.h:139-153) from events logged with kind
    EV_HISTORY: the moving atom's position after its flight at each displaced
    recoil, as an (n, 3) array sorted like the text streams."""
    h = _sorted(events[events["kind"] == F.EV_HISTORY])
    return np.stack([h["x"], h["y"], h["z"]], axis=1) if len(h) else np.zeros((0, 3))


def write(lines: Iterable[str], out: TextIO) -> int:
    n = 0
    for line in lines:
        out.write(line + "\n")
        n += 1
    return n


DEFECT_KINDS = (F.EV_VACANCY, F.EV_REST)
PHONON_KINDS = (F.EV_BRANCH, F.EV_DISSIPATE, F.EV_REST)
