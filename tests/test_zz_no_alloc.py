"""The allocation-free tally reduction, for hosts whose own allocator owns the
GPU's memory, gives the same totals as the regular run.

The tallies of a run are copied into device buffers that the test (standing in
for such a host) owns; mtg_reduce_primaries_noalloc reduces them through the C
ABI, twice in a row on different runs, and each result is compared with the
totals mtg_run reported.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _reduce_noalloc(lib, prim, stream):
    import torch
    dev = torch.device("cuda:0")
    bufs = {
        "vacancies": torch.from_numpy(prim["vacancies"].astype(np.uint64).view(np.int64)).to(dev),
        "collisions": torch.from_numpy(prim["collisions"].astype(np.uint64).view(np.int64)).to(dev),
        "eel": torch.from_numpy(prim["eel"]).to(dev),
        "enuc": torch.from_numpy(prim["enuc"]).to(dev),
        "x": torch.from_numpy(prim["x"]).to(dev),
        "y": torch.from_numpy(prim["y"]).to(dev),
        "z": torch.from_numpy(prim["z"]).to(dev),
        "state": torch.from_numpy(prim["state"]).to(dev),
    }
    out = torch.full((15,), float("nan"), dtype=torch.float64, device=dev)
    err = C.create_string_buffer(256)
    n = len(prim["eel"])
    p = lambda t: C.c_void_p(t.data_ptr())
    st = lib.mtg_reduce_primaries_noalloc(p(bufs["vacancies"]), p(bufs["collisions"]), p(bufs["eel"]),
                                          p(bufs["enuc"]), p(bufs["x"]), p(bufs["y"]), p(bufs["z"]),
                                          p(bufs["state"]), n, p(out), C.c_void_p(stream), err, len(err))
    assert st == 0, err.value.decode()
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _check(q, t):
    """the same bits: both reductions add the same numbers in the same order"""
    want = [t["vacancies"], t["vac_s2"], t["collisions"], t["coll_s2"], t["Eel"], t["eel_s2"], t["Enuc"],
            t["enuc_s2"], t["range_n"], t["sx"], t["sxx"], t["sy"], t["syy"], t["sz"], t["szz"]]
    for k, (a, b) in enumerate(zip(q, want)):
        assert float(a) == float(b), (k, a, b)


def test_noalloc_reduction_matches_run_totals(engine_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test without a CUDA device")
    from mytrim_gb300 import Engine
    from mytrim_gb300 import _ffi as F
    from mytrim_gb300 import workloads as W

    lib = F.load()
    stream = torch.cuda.current_stream().cuda_stream
    runs = [("fp64", W.cu_self_ion(n_primaries=2000, E=10e3), 5),
            ("fp32", W.arsenic_implant(n_primaries=70_000), 6)]
    for prec, sim, seed in runs:
        e = Engine(precision=prec, seed=seed)
        t = e.run([sim])[0]
        prim = e.primaries(0, sim.n_primaries)
        e.close()
        q = _reduce_noalloc(lib, prim, stream)
        _check(q, t)


def test_noalloc_rejects_oversized_input(engine_lib):
    from mytrim_gb300 import _ffi as F
    lib = F.load()
    err = C.create_string_buffer(256)
    one = C.c_void_p(16)  # never dereferenced: the size check comes first
    st = lib.mtg_reduce_primaries_noalloc(one, one, one, one, one, one, one, one, 65536 * 1024 + 1, one, None, err,
                                          len(err))
    assert st == 1
    assert b"exceed" in err.value
