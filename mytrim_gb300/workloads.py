"""The benchmark workloads: simulations described by their physical parameters.

Masses are the SRIM "MAI weight" column of the stopping tables for the ions and
the natural weights for targets; densities are the ones the workload names.
"""
import functools
import math

import numpy as np

from . import _ffi as F
from .engine import ElementSpec, LayerSpec, SimSpec

CU = 63.546
SI = 28.086
O = 15.999


def cu_self_ion(n_primaries=10_000, E=100e3):
    """Cu 100 keV normal incidence into bulk Cu (8.96 g/cm3, Edisp 25, Ebind 3, Ef 5 eV),
    full cascade, 1 nm range histogram to 200 nm."""
    return SimSpec(layers=[LayerSpec(1e7, 8.96, [ElementSpec(29, CU, 1.0, 25.0, 3.0)])],
                   Z=29, m=CU, E=E, Ef=5.0, n_primaries=n_primaries,
                   hist_range_bin=10.0, hist_range_n=200, hist_vac_bin=10.0, hist_vac_n=200)


def sio2_on_si(Z, m, E, n_primaries, tilt_deg=7.0):
    """Ion at `tilt_deg` into 10 nm SiO2 (2.2 g/cm3; Edisp Si 15, O 28) on bulk Si (2.33,
    Edisp 15); backscattered ions leave through the surface (CUT at x < 0);
    0.5 nm depth histogram to 300 nm, lateral 1 nm histogram over +-150 nm."""
    t = math.radians(tilt_deg)
    layers = [LayerSpec(100.0, 2.2, [ElementSpec(14, SI, 1.0, 15.0, 3.0), ElementSpec(8, O, 2.0, 28.0, 3.0)]),
              LayerSpec(1e7, 2.33, [ElementSpec(14, SI, 1.0, 15.0, 3.0)])]
    return SimSpec(layers=layers, Z=Z, m=m, E=E, n_primaries=n_primaries, dir=(math.cos(t), math.sin(t), 0.0),
                   pos=(0.0, 0.0, 0.0), size=(1e9, 1e9, 1e9), bc=(F.BC_CUT, F.BC_INF, F.BC_INF),
                   hist_range_bin=5.0, hist_range_n=600, hist_vac_bin=5.0, hist_vac_n=600,
                   hist_lateral_bin=10.0, hist_lateral_n=300)


def boron_implant(n_primaries=1_000_000):
    return sio2_on_si(5, 11.009, 10e3, n_primaries)


def arsenic_implant(n_primaries=1_000_000):
    return sio2_on_si(33, 74.922, 50e3, n_primaries)


def silver_into_silicon(n_primaries=10_000_000):
    """Ag 200 keV into bulk Si (2.33 g/cm3, Edisp 15, Ebind 3): the surrogate workload."""
    return SimSpec(layers=[LayerSpec(1e7, 2.33, [ElementSpec(14, SI, 1.0, 15.0, 3.0)])],
                   Z=47, m=106.905, E=200e3, n_primaries=n_primaries,
                   hist_range_bin=10.0, hist_range_n=300, hist_vac_bin=10.0, hist_vac_n=300)


def gold_deposition(n_primaries=100_000_000, voxels=256):
    """Au 1 MeV into 50 nm Ag / 200 nm Cu / bulk Si, full cascade, surface loss (CUT at
    x < 0) with sputter counting (E_surf 3 eV), energy deposition in voxels^3 cells over
    a 300 nm deep, 100 x 100 nm box around the beam, vacancy depth profile."""
    layers = [LayerSpec(500.0, 10.49, [ElementSpec(47, 107.868, 1.0)]),
              LayerSpec(2000.0, 8.96, [ElementSpec(29, CU, 1.0)]),
              LayerSpec(1e7, 2.33, [ElementSpec(14, SI, 1.0, 15.0, 3.0)])]
    return SimSpec(layers=layers, Z=79, m=196.967, E=1e6, n_primaries=n_primaries, pos=(0.0, 0.0, 0.0),
                   size=(1e9, 1e9, 1e9), bc=(F.BC_CUT, F.BC_INF, F.BC_INF),
                   hist_range_bin=10.0, hist_range_n=300, hist_vac_bin=10.0, hist_vac_n=300,
                   surface_binding=3.0, voxel_n=(voxels, voxels, voxels), voxel_origin=(0.0, -500.0, -500.0),
                   voxel_size=(3000.0, 1000.0, 1000.0))


def xenon_bubbles(n_primaries=1_000_000, n_bubbles=200, radius=15.0, box=400.0, seed=3):
    """Xe 30 keV into UO2 (10.97 g/cm3; Edisp U 40, O 20 eV) holding n_bubbles solid-Xe
    bubbles (3.5 g/cm3) of `radius` in a periodic box of edge `box` (sampleClusters,
    spatial hash of 19^3 cells): the cluster-geometry workload, full cascade.  Bubble
    centres are placed at random with at least 5 A between surfaces (the placement
    rule of sampleClusters::addRandomClusters, sample_clusters.C:228-250)."""
    cl = _bubbles(n_bubbles, radius, box, seed)
    uo2 = LayerSpec(box, 10.97, [ElementSpec(92, 238.03, 1.0, 40.0, 3.0), ElementSpec(8, O, 2.0, 20.0, 3.0)])
    xe = LayerSpec(box, 3.5, [ElementSpec(54, 131.29, 1.0, 25.0, 3.0)])
    return SimSpec(layers=[uo2, xe], Z=54, m=131.29, E=30e3, n_primaries=n_primaries,
                   pos=(0.0, box / 2, box / 2), size=(box, box, box), geometry="clusters",
                   clusters=cl, cluster_hash=(19, 19, 19), hist_range_bin=10.0, hist_range_n=200)


@functools.lru_cache(maxsize=8)
def _bubbles(n, radius, box, seed):
    rng = np.random.default_rng(seed)
    cl = []
    while len(cl) < n:
        q = rng.uniform(0.0, box, 3)
        ok = True
        for c in cl:
            d = q - c[:3]
            d -= np.round(d / box) * box
            if d @ d < (2 * radius + 5.0) ** 2:
                ok = False
                break
        if ok:
            cl.append(np.array([q[0], q[1], q[2], radius]))
    out = np.array(cl)
    out.setflags(write=False)
    return out


# targets of the batched workload: (name, rho, [(Z, mass, fraction, Edisp)])
TARGETS = [
    ("Si", 2.33, [(14, SI, 1.0, 15.0)]),
    ("Cu", 8.96, [(29, CU, 1.0, 25.0)]),
    ("Ag", 10.49, [(47, 107.868, 1.0, 25.0)]),
    ("Au", 19.32, [(79, 196.967, 1.0, 25.0)]),
    ("SiO2", 2.2, [(14, SI, 1.0, 15.0), (8, O, 2.0, 28.0)]),
    ("Al2O3", 3.95, [(13, 26.982, 2.0, 25.0), (8, O, 3.0, 28.0)]),
]


def srim_masses():
    """MAI weight (SCOEF.95A "m1" column) of Z = 1..92, the mass the batched workload gives each ion."""
    from .engine import TABLES
    out = []
    for line in TABLES.read_text().splitlines():
        if line.startswith("#") or not line.strip():
            continue
        out.append(float(line.split()[3]))
    return out


def batched_uneven(n_sims=4096, seed=1, scale_primaries=1.0, ion_masses=None):
    """4096 independent simulations drawn from `seed`: Z1 uniform 1..83 with the SRIM
    mass, E0 log-uniform 1 keV - 1 MeV, incidence angle uniform 0-60 deg, 1-4 layers
    from TARGETS with thickness log-uniform 5-500 nm over bulk Si, primaries
    log-uniform 1e2 - 1e5 (times `scale_primaries`)."""
    rng = np.random.default_rng(seed)
    if ion_masses is None:
        ion_masses = srim_masses()
    sims = []
    for _ in range(n_sims):
        Z = int(rng.integers(1, 84))
        m = ion_masses[Z - 1]
        E = float(10 ** rng.uniform(3, 6))
        ang = math.radians(float(rng.uniform(0, 60)))
        nl = int(rng.integers(1, 5))
        layers = []
        for _ in range(nl):
            name, rho, els = TARGETS[int(rng.integers(0, len(TARGETS)))]
            th = float(10 ** rng.uniform(math.log10(50.0), math.log10(5000.0)))
            layers.append(LayerSpec(th, rho, [ElementSpec(z, mm, f, ed, 3.0) for z, mm, f, ed in els]))
        layers.append(LayerSpec(1e7, 2.33, [ElementSpec(14, SI, 1.0, 15.0, 3.0)]))
        n = max(1, int(round(10 ** rng.uniform(2, 5) * scale_primaries)))
        sims.append(SimSpec(layers=layers, Z=Z, m=m, E=E, n_primaries=n,
                            dir=(math.cos(ang), math.sin(ang), 0.0), pos=(0.0, 0.0, 0.0),
                            size=(1e9, 1e9, 1e9), bc=(F.BC_CUT, F.BC_INF, F.BC_INF),
                            hist_range_bin=10.0, hist_range_n=100))
    return sims
