"""The small runs whose reference results are stored in ref_records.json.

Each case: (SimSpec, master seed, number of per-primary records kept).
"""
import math

import numpy as np

from mytrim_gb300.engine import ElementSpec, LayerSpec, SimSpec


def random_clusters(n, r, gap, box, seed):
    """n non-overlapping spheres of radius r, surfaces at least `gap` apart in a
    periodic box (the placement rule of sampleClusters::addRandomClusters,
    sample_clusters.C:228-250, with numpy's generator)."""
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n:
        p = rng.uniform(0.0, 1.0, 3) * np.asarray(box)
        ok = True
        for q in out:
            d = p - q[:3]
            d -= np.round(d / box) * box
            if d @ d < (2 * r + gap) ** 2:
                ok = False
                break
        if ok:
            out.append(np.array([p[0], p[1], p[2], r]))
    return np.array(out)

SI, O, CU = 28.086, 15.999, 63.546

CASES = {
    # runmytrim-style bulk copper (validation/vacancy_count/cu_on_cu_vac.json at 1 keV)
    "cu_1kev_vaccount": (SimSpec(layers=[LayerSpec(100000.0, 8.92, [ElementSpec(29, CU, 1.0)])], Z=29, m=CU,
                                 E=1000.0, n_primaries=60, hist_range_bin=10.0, hist_range_n=50,
                                 hist_vac_bin=1.0, hist_vac_n=60), 2344, 60),
    # tilted arsenic into SiO2 on Si with a CUT surface
    "as_sio2_si_cut": (SimSpec(layers=[LayerSpec(100.0, 2.2, [ElementSpec(14, SI, 1.0, 15.0, 3.0),
                                                              ElementSpec(8, O, 2.0, 28.0, 3.0)]),
                                       LayerSpec(100000.0, 2.33, [ElementSpec(14, SI, 1.0, 15.0, 3.0)])],
                               Z=33, m=74.922, E=20000.0, n_primaries=8, Ef=5.0,
                               dir=(math.cos(math.radians(7)), math.sin(math.radians(7)), 0.0),
                               pos=(0.0, 0.0, 0.0), size=(1e9, 1e9, 1e9), bc=(2, 1, 1),
                               hist_range_bin=5.0, hist_range_n=100, hist_vac_bin=5.0, hist_vac_n=100),
                       7, 8),
    # helium with TrimRange semantics (Kinchin-Pease vacancies, no recoils followed)
    "he_fe_range": (SimSpec(layers=[LayerSpec(100000.0, 7.8658, [ElementSpec(26, 55.847, 1.0)])], Z=2, m=4.0026,
                            E=20000.0, n_primaries=30, mode="range", hist_range_bin=10.0, hist_range_n=200),
                    11, 30),
    # gold into Ag / Cu / Si with a CUT surface, sputter counting and deposition voxels
    "au_agcusi_sputter": (SimSpec(layers=[LayerSpec(50.0, 10.49, [ElementSpec(47, 107.868, 1.0)]),
                                          LayerSpec(100.0, 8.96, [ElementSpec(29, CU, 1.0)]),
                                          LayerSpec(100000.0, 2.33, [ElementSpec(14, SI, 1.0, 15.0, 3.0)])],
                                  Z=79, m=196.967, E=20000.0, n_primaries=6, pos=(0.0, 0.0, 0.0),
                                  size=(1e9, 1e9, 1e9), bc=(2, 1, 1), surface_binding=3.0,
                                  voxel_n=(30, 4, 4), voxel_origin=(0.0, -100.0, -100.0),
                                  voxel_size=(300.0, 200.0, 200.0)), 5, 6),
    # xenon into UO2 holding xenon bubbles (sampleClusters, periodic 400 A box)
    "xe_uo2_clusters": (SimSpec(layers=[LayerSpec(400.0, 10.0, [ElementSpec(92, 235.0, 1.0), ElementSpec(8, 16.0, 2.0)]),
                                        LayerSpec(400.0, 3.5, [ElementSpec(54, 132.0, 1.0)])],
                                Z=54, m=132.0, E=30000.0, n_primaries=16, pos=(0.0, 200.0, 200.0),
                                size=(400.0, 400.0, 400.0), geometry="clusters",
                                clusters=random_clusters(40, 20.0, 25.0, (400.0, 400.0, 400.0), 3),
                                cluster_hash=(19, 19, 19), hist_range_bin=10.0, hist_range_n=100), 5, 16),
    # TrimPrimaries / TrimRecoils: generation cutoff 1 and 2 with the modified
    # Kinchin-Pease count at the cutoff (trim.C:446-464), into a two-element target
    "xe_sic_primaries": (SimSpec(layers=[LayerSpec(100000.0, 3.21, [ElementSpec(14, SI, 1.0, 35.0, 3.0),
                                                                     ElementSpec(6, 12.011, 1.0, 20.0, 3.0)])],
                                 Z=54, m=131.29, E=30000.0, n_primaries=30, mode="primaries", max_generation=1,
                                 hist_range_bin=10.0, hist_range_n=100), 17, 30),
    "xe_sic_recoils": (SimSpec(layers=[LayerSpec(100000.0, 3.21, [ElementSpec(14, SI, 1.0, 35.0, 3.0),
                                                                   ElementSpec(6, 12.011, 1.0, 20.0, 3.0)])],
                               Z=54, m=131.29, E=30000.0, n_primaries=30, mode="primaries", max_generation=2,
                               hist_range_bin=10.0, hist_range_n=100), 18, 30),
    # the other two potentials of TrimBase::_potential (trim.C:194-258)
    "cu_cu_moliere": (SimSpec(layers=[LayerSpec(100000.0, 8.92, [ElementSpec(29, CU, 1.0)])], Z=29, m=CU,
                              E=5000.0, n_primaries=30, potential="moliere", hist_range_bin=5.0,
                              hist_range_n=100), 21, 30),
    "kr_c_ckr": (SimSpec(layers=[LayerSpec(100000.0, 2.26, [ElementSpec(6, 12.011, 1.0, 28.0, 3.0)])], Z=36,
                         m=83.798, E=10000.0, n_primaries=30, potential="ckr", hist_range_bin=5.0,
                         hist_range_n=100), 22, 30),
    # protons into a two-element target
    "h_sic": (SimSpec(layers=[LayerSpec(100000.0, 3.21, [ElementSpec(14, SI, 1.0), ElementSpec(6, 12.011, 1.0)])],
                      Z=1, m=1.008, E=5000.0, n_primaries=40), 12, 40),
}
