"""Python front of the GB300 cascade engine (ctypes over include/mytrim_gpu.h).

``Engine`` owns one mtg_ctx.  ``SimSpec`` describes one simulation in the terms
of the reference's runmytrim input (layers of elements, an ion template, a
primary count and the tally options of apps/runmytrim.C:103-285).
"""
import ctypes as C
import math
from dataclasses import dataclass
from pathlib import Path
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _ffi as F

DATA_DIR = Path(__file__).resolve().parent / "data"
TABLES = DATA_DIR / "stopping_tables.tsv"

PRECISIONS = {"fp64": F.PREC_FP64, "fp32": F.PREC_FP32, "surrogate": F.PREC_FP32_SURROGATE}
# TrimBase::Potential (trim.h:63-69)
POTENTIALS = {"universal": F.POT_UNIVERSAL, "moliere": F.POT_MOLIERE, "ckr": F.POT_CKR}


@dataclass
class ElementSpec:
    Z: int
    m: float
    t: float = 1.0
    Edisp: float = 25.0  # Element defaults (element.C:25)
    Elbind: float = 3.0


@dataclass
class LayerSpec:
    thickness: float
    rho: float
    elements: List[ElementSpec]


@dataclass
class SimSpec:
    """One simulation: sample, ion template, primaries and tallies."""
    layers: List[LayerSpec]
    Z: int
    m: float
    E: float
    n_primaries: int
    Ef: float = 3.0                      # IonBase::_Ef default (ion.C:26)
    first_primary: int = 0               # primary index offset (sharded runs)
    dir: Tuple[float, float, float] = (1.0, 0.0, 0.0)
    pos: Optional[Tuple[float, float, float]] = None  # default (0, w1/2, w2/2) as runmytrim.C:298
    size: Optional[Tuple[float, float, float]] = None  # default (total thickness, 100, 100)
    bc: Tuple[int, int, int] = (F.BC_PBC, F.BC_PBC, F.BC_PBC)
    mode: str = "vaccount"               # or "range", or "primaries" (TrimPrimaries / TrimRecoils)
    max_generation: int = 1              # mode "primaries": TrimPrimaries::maxGen
    primaries_only: bool = False
    hist_range_bin: float = 10.0
    hist_range_n: int = 0
    hist_vac_bin: float = 1.0
    hist_vac_n: int = 0
    surface_binding: float = 0.0         # sputter counting (extension), 0 = off
    voxel_n: Tuple[int, int, int] = (0, 0, 0)  # energy-deposition voxels (extension)
    voxel_origin: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    voxel_size: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    hist_lateral_bin: float = 10.0       # lateral (y, z) histogram of stopping points
    hist_lateral_n: int = 0
    hist_evac_rows: int = 0              # vacancy-energy histogram rows (int(ln E))
    potential: str = "universal"         # TrimBase::_potential: "universal", "moliere" or "ckr"
    # IonMDTag::_md as the reference's demo programs mark it (apps/mytrim_solid.C:156-159):
    # members of atomic number md_tag_Z starting with an energy inside md_tag_E get
    # _md = 1 in the event log; 0 = off
    md_tag_Z: int = 0
    md_tag_E: Tuple[float, float] = (200.0, 12000.0)
    # sampleClusters geometry: layers[0] is the matrix, layers[1] the cluster
    # material; clusters is an (n, 4) array of x, y, z, r; cluster_hash the
    # spatial-hash cells per axis (sampleClusters::initSpatialhash)
    geometry: str = "layers"
    clusters: Optional[np.ndarray] = None
    cluster_hash: Tuple[int, int, int] = (1, 1, 1)

    def box(self):
        if self.size is not None:
            return tuple(self.size)
        return (sum(l.thickness for l in self.layers), 100.0, 100.0)

    def start(self):
        if self.pos is not None:
            return tuple(self.pos)
        w = self.box()
        return (0.0, w[1] / 2.0, w[2] / 2.0)

    def hist_sizes(self):
        evac = self.hist_evac_rows * self.hist_vac_n if self.hist_vac_n > 0 else 0
        return self.hist_range_n, self.hist_vac_n, self.hist_vac_n, self.hist_lateral_n ** 2, evac

    def to_c(self) -> F.Sim:
        if not 1 <= len(self.layers) <= F.MAX_LAYERS:
            raise ValueError("1 to 8 layers")
        s = F.Sim()
        s.sample.n_layers = len(self.layers)
        for i, l in enumerate(self.layers):
            s.sample.thickness[i] = l.thickness
            s.sample.material[i] = _c_material(l)
        s.sample.w[0:3] = self.box()
        s.sample.bc[0:3] = self.bc
        if self.geometry == "clusters":
            if len(self.layers) != 2:
                raise ValueError("a cluster sample needs two materials (matrix, cluster)")
            cl = np.ascontiguousarray(self.clusters if self.clusters is not None else np.zeros((0, 4)),
                                      dtype=np.float64).reshape(-1, 4)
            s.sample.geometry = F.GEOM_CLUSTERS
            for i in range(3):
                s.sample.cluster_hash[i] = int(self.cluster_hash[i])
            s.sample.n_clusters = len(cl)
            s.sample.clusters = cl.ctypes.data_as(C.POINTER(C.c_double))
            s._keep = cl  # the array must outlive the call that reads it
        elif self.geometry != "layers":
            raise ValueError("geometry is 'layers' or 'clusters'")
        s.ion.Z = self.Z
        s.ion.m = self.m
        s.ion.E = self.E
        s.ion.Ef = self.Ef
        s.ion.dir[0:3] = self.dir
        s.ion.pos[0:3] = self.start()
        s.n_primaries = self.n_primaries
        s.first_primary = self.first_primary
        s.tally_mode = {"vaccount": F.TALLY_VACCOUNT, "range": F.TALLY_RANGE,
                        "primaries": F.TALLY_PRIMARIES}[self.mode]
        s.max_generation = self.max_generation
        s.primaries_only = int(self.primaries_only)
        s.hist_range_bin = self.hist_range_bin
        s.hist_range_n = self.hist_range_n
        s.hist_vac_bin = self.hist_vac_bin
        s.hist_vac_n = self.hist_vac_n
        s.surface_binding = self.surface_binding
        s.hist_lateral_bin = self.hist_lateral_bin
        s.hist_lateral_n = self.hist_lateral_n
        s.hist_evac_rows = self.hist_evac_rows
        s.potential = POTENTIALS[self.potential]
        s.md_tag_Z = self.md_tag_Z
        s.md_tag_Emin, s.md_tag_Emax = self.md_tag_E
        s.voxel_n[0:3] = self.voxel_n
        s.voxel_origin[0:3] = self.voxel_origin
        s.voxel_size[0:3] = self.voxel_size
        return s


# mtg_material structs by value: batches of many simulations reuse a few materials
_MATERIALS: dict = {}
_MAT_BYTES: dict = {}


class _SampleRow(C.Structure):
    # mtg_sample with the cluster pointer as an integer (a numpy dtype needs that)
    _fields_ = [(n, C.c_uint64 if n == "clusters" else t) for n, t in F.Sample._fields_]


class _SimRow(C.Structure):
    _fields_ = [(n, _SampleRow if n == "sample" else t) for n, t in F.Sim._fields_]


_SIM_DTYPE = np.dtype(_SimRow)
assert _SIM_DTYPE.itemsize == C.sizeof(F.Sim)
_NO_MATERIAL = bytes(C.sizeof(F.Material))
_TALLY_MODES = {"vaccount": F.TALLY_VACCOUNT, "range": F.TALLY_RANGE, "primaries": F.TALLY_PRIMARIES}


def sims_to_array(sims: Sequence["SimSpec"]):
    """The mtg_sim array of a run as a numpy structured array with the same bytes
    as SimSpec.to_c() of each simulation, filled column by column (a batch of
    thousands of simulations converts in milliseconds).  Returns the array and the
    objects that must outlive the call reading it (cluster lists)."""
    n = len(sims)
    a = np.zeros(n, _SIM_DTYPE)
    keep = []
    mats = []
    thick = np.zeros((n, F.MAX_LAYERS))
    for k, s in enumerate(sims):
        nl = len(s.layers)
        if not 1 <= nl <= F.MAX_LAYERS:
            raise ValueError("1 to 8 layers")
        for i, l in enumerate(s.layers):
            thick[k, i] = l.thickness
            mats.append(_material_bytes(l))
        mats.append(_NO_MATERIAL * (F.MAX_LAYERS - nl))
        if s.geometry == "clusters":
            if nl != 2:
                raise ValueError("a cluster sample needs two materials (matrix, cluster)")
            cl = np.ascontiguousarray(s.clusters if s.clusters is not None else np.zeros((0, 4)),
                                      dtype=np.float64).reshape(-1, 4)
            keep.append(cl)
            a["sample"]["geometry"][k] = F.GEOM_CLUSTERS
            a["sample"]["cluster_hash"][k] = [int(v) for v in s.cluster_hash]
            a["sample"]["n_clusters"][k] = len(cl)
            a["sample"]["clusters"][k] = cl.ctypes.data
        elif s.geometry != "layers":
            raise ValueError("geometry is 'layers' or 'clusters'")
    smp = a["sample"]
    smp["n_layers"] = [len(s.layers) for s in sims]
    smp["thickness"] = thick
    smp["material"] = np.frombuffer(b"".join(mats), dtype=smp.dtype["material"].base).reshape(n, F.MAX_LAYERS)
    smp["w"] = [s.box() for s in sims]
    smp["bc"] = [s.bc for s in sims]
    ion = a["ion"]
    ion["Z"] = [s.Z for s in sims]
    ion["m"] = [s.m for s in sims]
    ion["E"] = [s.E for s in sims]
    ion["Ef"] = [s.Ef for s in sims]
    ion["dir"] = [s.dir for s in sims]
    ion["pos"] = [s.start() for s in sims]
    a["n_primaries"] = [s.n_primaries for s in sims]
    a["first_primary"] = [s.first_primary for s in sims]
    a["tally_mode"] = [_TALLY_MODES[s.mode] for s in sims]
    a["max_generation"] = [s.max_generation for s in sims]
    a["primaries_only"] = [int(s.primaries_only) for s in sims]
    for f in ("hist_range_bin", "hist_range_n", "hist_vac_bin", "hist_vac_n", "surface_binding",
              "hist_lateral_bin", "hist_lateral_n", "hist_evac_rows", "voxel_n", "voxel_origin", "voxel_size"):
        a[f] = [getattr(s, f) for s in sims]
    a["potential"] = [POTENTIALS[s.potential] for s in sims]
    a["md_tag_Z"] = [s.md_tag_Z for s in sims]
    a["md_tag_Emin"] = [s.md_tag_E[0] for s in sims]
    a["md_tag_Emax"] = [s.md_tag_E[1] for s in sims]
    return a, keep


def _material_bytes(l: "LayerSpec") -> bytes:
    key = (l.rho, tuple((e.Z, e.m, e.t, e.Edisp, e.Elbind) for e in l.elements))
    b = _MAT_BYTES.get(key)
    if b is None:
        b = bytes(_c_material(l))
        if len(_MAT_BYTES) > 4096:
            _MAT_BYTES.clear()
        _MAT_BYTES[key] = b
    return b


def _c_material(l: "LayerSpec") -> F.Material:
    if not 1 <= len(l.elements) <= F.MAX_ELEMENTS:
        raise ValueError("1 to 4 elements per layer")
    key = (l.rho, tuple((e.Z, e.m, e.t, e.Edisp, e.Elbind) for e in l.elements))
    mat = _MATERIALS.get(key)
    if mat is None:
        mat = F.Material()
        mat.rho = l.rho
        mat.n_elements = len(l.elements)
        for j, e in enumerate(l.elements):
            mat.elements[j].Z = e.Z
            mat.elements[j].m = e.m
            mat.elements[j].t = e.t
            mat.elements[j].Edisp = e.Edisp
            mat.elements[j].Elbind = e.Elbind
        if len(_MATERIALS) > 4096:
            _MATERIALS.clear()
        _MATERIALS[key] = mat
    return mat


def summarize(t: dict) -> dict:
    """Per-ion statistics with standard errors from the per-primary moments."""
    n = max(t["primaries"], 1)
    out = dict(t)

    def mean_err(s1, s2, count):
        if count <= 0:
            return float("nan"), float("nan")
        m = s1 / count
        var = max(s2 / count - m * m, 0.0)
        return m, math.sqrt(var / max(count - 1, 1))

    out["vac_per_ion"], out["vac_per_ion_err"] = mean_err(t["vacancies"], t["vac_s2"], n)
    out["eel_per_ion"], out["eel_per_ion_err"] = mean_err(t["Eel"], t["eel_s2"], n)
    out["enuc_per_ion"], out["enuc_per_ion_err"] = mean_err(t["Enuc"], t["enuc_s2"], n)
    out["coll_per_ion"], out["coll_per_ion_err"] = mean_err(t["collisions"], t["coll_s2"], n)
    rn = t["range_n"]
    if rn > 1:
        mx = t["sx"] / rn
        vx = max(t["sxx"] / rn - mx * mx, 0.0)
        my, mz = t["sy"] / rn, t["sz"] / rn
        vy = max(t["syy"] / rn - my * my, 0.0)
        vz = max(t["szz"] / rn - mz * mz, 0.0)
        out["range_mean"] = mx
        out["range_mean_err"] = math.sqrt(vx / (rn - 1))
        out["straggle"] = math.sqrt(vx)
        # standard error of a standard deviation (normal approximation)
        out["straggle_err"] = math.sqrt(vx) / math.sqrt(2.0 * (rn - 1))
        out["lateral"] = math.sqrt(vy + vz)
        out["lateral_err"] = math.sqrt(vy + vz) / math.sqrt(2.0 * (rn - 1))
    return out


class Engine:
    """One engine context on one GPU."""

    def __init__(self, device: int = 0, precision: str = "fp64", seed: int = 1, tmin: float = 0.2,
                 tau: float = 0.0, cw: float = 0.001, length_scale: float = 1.0, max_collisions: int = 0,
                 stack_capacity: int = 0, tables: Optional[str] = None, block_threads: int = 0,
                 max_take: int = 0):
        self.lib = F.load()
        self.ctx = C.c_void_p()
        st = self.lib.mtg_create(device, C.byref(self.ctx))
        if st != F.OK:
            raise F.EngineError(st, "mtg_create failed")
        self._check(self.lib.mtg_load_tables(self.ctx, str(tables or TABLES).encode()))
        self.cfg = F.Config()
        self.configure(precision=precision, seed=seed, tmin=tmin, tau=tau, cw=cw, length_scale=length_scale,
                       max_collisions=max_collisions, stack_capacity=stack_capacity, block_threads=block_threads,
                       max_take=max_take)
        self._sims: List[SimSpec] = []

    def _check(self, st):
        if st != F.OK:
            msg = self.lib.mtg_last_error(self.ctx)
            raise F.EngineError(st, msg.decode() if msg else "")
        return st

    def configure(self, precision="fp64", seed=1, tmin=0.2, tau=0.0, cw=0.001, length_scale=1.0,
                  max_collisions=0, stack_capacity=0, block_threads=0, max_take=0, refill_min_idle=0):
        c = self.cfg
        c.tmin, c.tau, c.cw, c.length_scale = tmin, tau, cw, length_scale
        c.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        c.seed = seed
        c.max_collisions_per_member = max_collisions
        c.stack_capacity = stack_capacity
        c.block_threads = block_threads
        c.max_primaries_per_refill = max_take
        c.refill_min_idle = refill_min_idle
        self._check(self.lib.mtg_configure(self.ctx, C.byref(c)))

    def close(self):
        if self.ctx:
            self.lib.mtg_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- runs
    def prepare(self, sims: Sequence[SimSpec]):
        arr, keep = sims_to_array(sims)
        self._sims = list(sims)
        self._check(self.lib.mtg_prepare(self.ctx, arr.ctypes.data_as(C.POINTER(F.Sim)), len(sims)))
        del keep  # held until here: cluster arrays are read during mtg_prepare

    def launch(self, stream: Optional[int] = None):
        self._check(self.lib.mtg_launch_async(self.ctx, C.c_void_p(stream or 0)))

    def collect(self, check=True, allow_event_overflow=False):
        """Wait for the launched run and return one tally dict per sim.  With
        allow_event_overflow a run whose only error was a full event log returns its
        (complete) tallies; stats()["events_overflowed"] then reads 1."""
        n = len(self._sims)
        tot = (F.Totals * n)()
        nh = sum(sum(s.hist_sizes()) for s in self._sims)
        hist = (C.c_longlong * max(nh, 1))()
        st = self.lib.mtg_collect(self.ctx, tot, hist)
        if check and not (allow_event_overflow and st == F.ERR_QUEUE_FULL and self.stats()["events_overflowed"]):
            self._check(st)
        out = []
        off = 0
        rows = np.ctypeslib.as_array(tot).tolist()
        names = F.Totals.field_names()
        h = np.frombuffer(hist, dtype=np.int64, count=max(nh, 1))
        for i, s in enumerate(self._sims):
            d = dict(zip(names, rows[i]))
            hr, hv, hp, hl, he = s.hist_sizes()
            d["hist_range"] = h[off:off + hr].copy()
            d["hist_vac"] = h[off + hr:off + hr + hv].copy()
            d["hist_repl"] = h[off + hr + hv:off + hr + hv + hp].copy()
            o = off + hr + hv + hp
            d["hist_lateral"] = h[o:o + hl].copy().reshape(s.hist_lateral_n, s.hist_lateral_n)
            d["hist_evac"] = h[o + hl:o + hl + he].copy().reshape(s.hist_evac_rows if he else 0, hv if he else 0)
            off += hr + hv + hp + hl + he
            d["status"] = st
            out.append(d)
        return out

    def run(self, sims: Sequence[SimSpec], check=True, allow_event_overflow=False):
        self.prepare(sims)
        self.launch()
        return self.collect(check=check, allow_event_overflow=allow_event_overflow)

    def primaries(self, first: int, n: int) -> dict:
        out = {k: np.zeros(n, dtype=np.int64) for k in ("vacancies", "collisions")}
        out.update({k: np.zeros(n, dtype=np.float64) for k in ("eel", "enuc", "x", "y", "z")})
        out["state"] = np.zeros(n, dtype=np.int32)
        p = lambda a, t: a.ctypes.data_as(C.POINTER(t))
        self._check(self.lib.mtg_get_primaries(
            self.ctx, first, n, p(out["vacancies"], C.c_longlong), p(out["collisions"], C.c_longlong),
            p(out["eel"], C.c_double), p(out["enuc"], C.c_double), p(out["x"], C.c_double),
            p(out["y"], C.c_double), p(out["z"], C.c_double), p(out["state"], C.c_int)))
        return out

    def voxels(self, sim: int = 0, fp64: bool = False) -> np.ndarray:
        """Energy-deposition voxels of simulation `sim` [eV], (nz, ny, nx): the FP32
        tally, or with fp64 the FP64 cell totals it is rounded from."""
        s = self._sims[sim]
        nx, ny, nz = s.voxel_n
        if fp64:
            out = np.zeros(nx * ny * nz, dtype=np.float64)
            self._check(self.lib.mtg_get_voxels64(self.ctx, sim, out.ctypes.data_as(C.POINTER(C.c_double)),
                                                  len(out)))
        else:
            out = np.zeros(nx * ny * nz, dtype=np.float32)
            self._check(self.lib.mtg_get_voxels(self.ctx, sim, out.ctypes.data_as(C.POINTER(C.c_float)), len(out)))
        return out.reshape(nz, ny, nx)

    def set_record_capacity(self, cap: int):
        self._check(self.lib.mtg_set_record_capacity(self.ctx, cap))
        self._record_cap = cap

    def records(self) -> np.ndarray:
        cap = getattr(self, "_record_cap", 0)
        buf = (F.MemberRecord * max(cap, 1))()
        n = C.c_longlong(0)
        self._check(self.lib.mtg_get_records(self.ctx, buf, cap, C.byref(n)))
        dt = np.dtype([("key", "<u8"), ("sim", "<i4"), ("species", "<i4"), ("gen", "<i4"), ("state", "<i4"),
                       ("ncoll", "<u4"), ("nvac", "<u4"), ("E", "<f8"), ("x", "<f8"), ("y", "<f8"),
                       ("z", "<f8"), ("eel", "<f8")])
        assert dt.itemsize == C.sizeof(F.MemberRecord)
        return np.frombuffer(bytes(buf)[: n.value * dt.itemsize], dtype=dt).copy()

    def set_event_log(self, kinds, capacity: int):
        """Log events of the given kinds (F.EV_* numbers) in subsequent runs."""
        mask = 0
        for k in kinds:
            mask |= 1 << int(k)
        self._check(self.lib.mtg_set_event_log(self.ctx, mask, capacity))
        self._event_cap = capacity if mask else 0

    def event_count(self) -> int:
        """Events the last run logged (may exceed the log's capacity)."""
        n, total = C.c_longlong(0), C.c_longlong(0)
        self._check(self.lib.mtg_get_events(self.ctx, None, 0, C.byref(n), C.byref(total)))
        return total.value

    def events(self) -> np.ndarray:
        """The last run's event records as a structured array (unordered)."""
        cap = getattr(self, "_event_cap", 0)
        dt = np.dtype([("x", "<f8"), ("y", "<f8"), ("z", "<f8"), ("E", "<f8"), ("aux", "<f8"), ("m", "<f8"), ("key", "<u8"),
                       ("primary", "<i8"), ("sim", "<i4"), ("kind", "<i4"), ("Z", "<i4"), ("gen", "<i4"),
                       ("state", "<i4"), ("tag", "<i4"), ("md", "<i4"), ("pad", "<i4")])
        assert dt.itemsize == C.sizeof(F.Event)
        want = min(cap, self.event_count())  # the records logged, at most the capacity
        out = np.zeros(max(want, 1), dtype=dt)
        n, total = C.c_longlong(0), C.c_longlong(0)
        self._check(self.lib.mtg_get_events(self.ctx, out.ctypes.data_as(C.POINTER(F.Event)), want, C.byref(n),
                                            C.byref(total)))
        return out[: n.value].copy()

    def stopping(self, Z1, m1, layer: LayerSpec, energies, precision="fp64") -> np.ndarray:
        e = np.ascontiguousarray(energies, dtype=np.float64)
        out = np.zeros_like(e)
        mat = SimSpec([layer], Z1, m1, 1.0, 0).to_c().sample.material[0]
        prec = PRECISIONS[precision] if isinstance(precision, str) else precision
        self._check(self.lib.mtg_stopping(self.ctx, Z1, m1, C.byref(mat), e.ctypes.data_as(C.POINTER(C.c_double)),
                                          len(e), prec, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def scatter(self, eps, b, precision="fp64", potential="universal") -> np.ndarray:
        e = np.ascontiguousarray(eps, dtype=np.float64)
        bb = np.ascontiguousarray(b, dtype=np.float64)
        out = np.zeros_like(e)
        prec = PRECISIONS[precision] if isinstance(precision, str) else precision
        pot = POTENTIALS[potential] if isinstance(potential, str) else potential
        pd = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        self._check(self.lib.mtg_scatter_potential(self.ctx, pd(e), pd(bb), len(e), prec, pot, pd(out)))
        return out

    # ---- learned scattering surrogate
    def surrogate_train(self, n_train=20_000_000, batch=16384, epochs=12, qat_epochs=2, lr=2e-3, seed=1,
                        w_tau=0.1, target="quadrature", weighting="uniform") -> dict:
        """Train the network; target "quadrature" (the true scattering integral) or
        "magic" (the magic formula the plain path evaluates, at the same samples);
        weighting "uniform" or "transfer" (each sample's error weighted by its
        sin^2(theta/2))."""
        cfg = F.SurrogateConfig(n_train, batch, epochs, qat_epochs, lr, seed, w_tau, F.SURROGATE_TARGETS[target],
                                F.SURROGATE_WEIGHTS[weighting])
        rep = F.SurrogateReport()
        self._check(self.lib.mtg_surrogate_train(self.ctx, C.byref(cfg), C.byref(rep)))
        return {"final_loss": rep.final_loss, "train_seconds": rep.train_seconds, "steps": rep.steps}

    def surrogate_params(self) -> np.ndarray:
        out = np.zeros(F.SURROGATE_NPARAM, dtype=np.float32)
        self._check(self.lib.mtg_surrogate_get_params(self.ctx, out.ctypes.data_as(C.POINTER(C.c_float)), len(out)))
        return out

    def set_surrogate_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.float32)
        self._check(self.lib.mtg_surrogate_set_params(self.ctx, p.ctypes.data_as(C.POINTER(C.c_float)), len(p)))

    def surrogate_gradients(self, params, x, y, w_tau=0.1):
        p = np.ascontiguousarray(params, dtype=np.float32)
        xx = np.ascontiguousarray(x, dtype=np.float32)
        yy = np.ascontiguousarray(y, dtype=np.float32)
        g = np.zeros(F.SURROGATE_NPARAM, dtype=np.float32)
        loss = C.c_float(0.0)
        pf = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        self._check(self.lib.mtg_surrogate_gradients(self.ctx, pf(p), pf(xx), pf(yy), len(xx), w_tau, C.byref(loss),
                                                     pf(g)))
        return loss.value, g

    def quadrature(self, eps, b):
        e = np.ascontiguousarray(eps, dtype=np.float64)
        bb = np.ascontiguousarray(b, dtype=np.float64)
        s2 = np.zeros_like(e)
        tau = np.zeros_like(e)
        pd = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        self._check(self.lib.mtg_surrogate_quadrature(self.ctx, pd(e), pd(bb), len(e), pd(s2), pd(tau)))
        return s2, tau

    def autotune(self, sims: Sequence[SimSpec], trial_primaries: int = 0) -> dict:
        """Choose the launch settings (refill size, block shape, stack depth) for runs
        like `sims` by timing trial launches (mtg_autotune); the context keeps them."""
        arr, keep = sims_to_array(sims)
        t = F.Tuning()
        self._check(self.lib.mtg_autotune(self.ctx, arr.ctypes.data, len(sims), trial_primaries, C.byref(t)))
        del keep
        if t.changed:  # keep the front end's copy of the configuration in step
            self.cfg.block_threads = t.block_threads
            self.cfg.max_primaries_per_refill = t.max_primaries_per_refill
            self.cfg.stack_capacity = t.stack_capacity
            self.cfg.refill_min_idle = t.refill_min_idle
        return {n: getattr(t, n) for n, _ in t._fields_}

    def stats(self) -> dict:
        s = F.Stats()
        self._check(self.lib.mtg_get_stats(self.ctx, C.byref(s)))
        return {n: getattr(s, n) for n, _ in s._fields_}
