"""The small runs whose reference results are stored in ref_records.json.

Each case: (SimSpec, master seed, number of per-primary records kept).
"""
import math

from mytrim_gb300.engine import ElementSpec, LayerSpec, SimSpec

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
    # protons into a two-element target
    "h_sic": (SimSpec(layers=[LayerSpec(100000.0, 3.21, [ElementSpec(14, SI, 1.0), ElementSpec(6, 12.011, 1.0)])],
                      Z=1, m=1.008, E=5000.0, n_primaries=40), 12, 40),
}
