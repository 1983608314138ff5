"""Reference-shaped API: the classes of MyTRIM's C++ interface, backed by the GPU engine.

A user of the reference builds a SimconfType, MaterialBase objects from Elements,
a SampleSolid / SampleLayers, an IonBase template and a TrimBase subclass, then
loops over primaries (apps/runmytrim.C:121-304).  The same objects exist here
with the same field names; ``TrimGPU.runPrimaries`` replaces the per-primary
FIFO loop of runmytrim.C:71-93 with one batched GPU run.  The C++ header
mytrim_gb300/cpp/trim_gpu.h offers the same classes to C++ callers.
"""
from typing import List, Optional

from . import _ffi as F
from .engine import ElementSpec, Engine, LayerSpec, SimSpec, summarize


class SimconfType:
    """Run-wide settings (simconf.h:47-128): tmin, tau, cw, length scale, seed."""

    def __init__(self, seed: int = 12345678):
        self._seed = seed
        self.tmin = 0.2  # runmytrim.C:126
        self.tau = 0.0
        self.cw = 0.001
        self._length_scale = 1.0
        self.EelTotal = 0.0
        self.EnucTotal = 0.0
        self.vacancies_created = 0

    def seed(self, s: int):
        self._seed = s

    def setLengthScale(self, l: float):
        self._length_scale = l

    def lengthScale(self) -> float:
        return self._length_scale


class Element:
    """Element (element.h:29-41)."""

    def __init__(self, Z: int = 1, m: float = 1.0, t: float = 1.0, Edisp: float = 25.0, Elbind: float = 3.0):
        self._Z, self._m, self._t, self._Edisp, self._Elbind = Z, m, t, Edisp, Elbind


class MaterialBase:
    """MaterialBase (material.h:34-75); rho in g/cm^3."""

    def __init__(self, simconf: SimconfType, rho: float):
        self._simconf = simconf
        self._rho = rho
        self._element: List[Element] = []

    def prepare(self):
        # normalisation happens in the engine's table setup (material.C:37-74)
        if not self._element or sum(max(e._t, 0.0) for e in self._element) <= 0.0:
            raise ValueError("Stoichiometry invalid, all elements zero.")

    def _layer(self, thickness: float) -> LayerSpec:
        return LayerSpec(thickness, self._rho,
                         [ElementSpec(e._Z, e._m, e._t, e._Edisp, e._Elbind) for e in self._element])


class SampleBase:
    PBC, INF, CUT = F.BC_PBC, F.BC_INF, F.BC_CUT

    def __init__(self, x: float = 10000.0, y: float = 10000.0, z: float = 10000.0):
        self.w = [x, y, z]
        self.bc = [self.PBC, self.PBC, self.PBC]  # sample.C:27-32
        self.material: List[MaterialBase] = []


class SampleSolid(SampleBase):
    """One material everywhere (sample_solid.C:26-29)."""

    def _layers(self):
        return [self.material[0]._layer(self.w[0])]


class SampleLayers(SampleBase):
    """Layers along x; x < 0 is layer 0, the last layer extends to +inf (sample_layers.C:27-43)."""

    def __init__(self, x: float, y: float, z: float):
        super().__init__(x, y, z)
        self.layerThickness: List[float] = []

    def _layers(self):
        return [m._layer(t) for m, t in zip(self.material, self.layerThickness)]


class sampleClusters(SampleBase):
    """Spheres of material[1] in a matrix of material[0] (sample_clusters.h:30-57),
    found through a spatial hash of initSpatialhash(x, y, z) cells."""

    def __init__(self, x: float, y: float, z: float):
        super().__init__(x, y, z)
        self.kn = [1, 1, 1]
        self.c: List[List[float]] = [[], [], [], []]  # x, y, z, r per cluster

    def initSpatialhash(self, x: int, y: int, z: int):
        self.kn = [int(x), int(y), int(z)]

    def addCluster(self, x: float, y: float, z: float, r: float):
        for v, lst in zip((x, y, z, r), self.c):
            lst.append(float(v))

    @property
    def cn(self) -> int:
        return len(self.c[0])

    def _layers(self):
        if len(self.material) != 2:
            raise ValueError("a cluster sample needs two materials (matrix, cluster)")
        return [m._layer(self.w[0]) for m in self.material]

    def _cluster_array(self):
        import numpy as np
        return np.array(self.c, dtype=np.float64).T.reshape(-1, 4)


class IonBase:
    """Ion template (ion.h:30-85)."""

    def __init__(self, Z: int = 1, m: float = 1.0, E: float = 0.0):
        self._Z, self._m, self._E = Z, m, E
        self._Ef = 3.0
        self._gen = 0
        self._dir = [1.0, 0.0, 0.0]
        self._pos: Optional[List[float]] = None


class TrimGPU:
    """Drop-in for a runmytrim TrimBase subclass (TrimVacCount / TrimRange /
    TrimPrimaries / TrimRecoils with TrimPhononOut energy accounting), running every
    primary's full cascade on the GPU.  ``output`` is "vaccount", "range" or
    "primaries" (with ``max_generation`` 1 for TrimPrimaries, 2 for TrimRecoils)."""

    # TrimBase::Potential (trim.h:63-69); assign one to _potential
    UNIVERSAL, MOLIERE, CKR = 0, 1, 2

    def __init__(self, simconf: SimconfType, sample: SampleBase, precision: str = "fp64", device: int = 0,
                 output: str = "vaccount", primaries_only: bool = False, max_generation: int = 1):
        if not isinstance(sample, (SampleSolid, SampleLayers, sampleClusters)):
            raise TypeError("TrimGPU supports SampleSolid, SampleLayers and sampleClusters")
        self._simconf = simconf
        self._sample = sample
        self._potential = self.UNIVERSAL
        self._output = output
        self._primaries_only = primaries_only
        self._max_generation = max_generation
        self._engine = Engine(device=device, precision=precision, seed=simconf._seed, tmin=simconf.tmin,
                              tau=simconf.tau, cw=simconf.cw, length_scale=simconf.lengthScale())

    def _spec(self, sample: SampleBase, pka: IonBase, n: int, hist_range, hist_vac) -> SimSpec:
        extra = {}
        if isinstance(sample, sampleClusters):
            extra = dict(geometry="clusters", clusters=sample._cluster_array(), cluster_hash=tuple(sample.kn))
        return SimSpec(layers=sample._layers(), Z=pka._Z, m=pka._m, E=pka._E, n_primaries=n, Ef=pka._Ef,
                       dir=tuple(pka._dir), pos=tuple(pka._pos) if pka._pos else None, size=tuple(sample.w),
                       bc=tuple(sample.bc), mode=self._output, max_generation=self._max_generation,
                       primaries_only=self._primaries_only, hist_range_bin=hist_range[0],
                       hist_range_n=hist_range[1], hist_vac_bin=hist_vac[0], hist_vac_n=hist_vac[1],
                       potential=("universal", "moliere", "ckr")[self._potential], **extra)

    def _account(self, r: dict):
        sc = self._simconf
        sc.EelTotal += r["Eel"]
        sc.EnucTotal += r["Enuc"]
        sc.vacancies_created += r["vacancies"]

    def runPrimaries(self, pka: IonBase, n: int, hist_range=(10.0, 0), hist_vac=(1.0, 0)) -> dict:
        r = self._engine.run([self._spec(self._sample, pka, n, hist_range, hist_vac)])[0]
        self._account(r)
        return summarize(r)

    def runBatch(self, jobs, hist_range=(10.0, 0), hist_vac=(1.0, 0)) -> list:
        """Several independent simulations in one launch: jobs of (sample, pka, n)."""
        specs = [self._spec(smp, pka, n, hist_range, hist_vac) for smp, pka, n in jobs]
        out = []
        for r in self._engine.run(specs):
            self._account(r)
            out.append(summarize(r))
        return out
