"""The C ABI library loads and exports every entry point include/mytrim_gpu.h
declares (no compute: these run without a GPU)."""
import re
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "mytrim_gpu.h"


def declared():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"\b(mtg_[a-z0-9_]+)\s*\(", text)))


def test_header_declarations_are_exported(engine_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(engine_lib)], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r" T (mtg_\w+)", out))
    names = declared()
    assert len(names) >= 16
    missing = [n for n in names if n not in exported]
    assert not missing, missing


def test_python_mirror_covers_header(engine_lib):
    from mytrim_gb300 import _ffi as F
    assert sorted(F.SIGNATURES) == declared()
    lib = F.load()
    for name in declared():
        assert hasattr(lib, name)


def test_struct_layouts_match_header(engine_lib, tmp_path):
    """sizeof of every public struct in C equals the ctypes mirror."""
    from mytrim_gb300 import _ffi as F
    structs = {"mtg_scoef_row": F.ScoefRow, "mtg_element": F.Element, "mtg_material": F.Material,
               "mtg_sample": F.Sample, "mtg_ion": F.Ion, "mtg_sim": F.Sim, "mtg_config": F.Config,
               "mtg_totals": F.Totals, "mtg_member_record": F.MemberRecord, "mtg_stats": F.Stats}
    src = tmp_path / "sz.c"
    src.write_text('#include "mytrim_gpu.h"\n#include <stdio.h>\nint main(void){\n' +
                   "".join(f'printf("%zu\\n", sizeof({n}));\n' for n in structs) + "return 0;}\n")
    exe = tmp_path / "sz"
    subprocess.run(["gcc", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], check=True)
    sizes = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    import ctypes
    for (n, cls), sz in zip(structs.items(), sizes):
        assert ctypes.sizeof(cls) == sz, n


def test_create_without_device_fails_cleanly(engine_lib):
    """No GPU here: mtg_create reports MTG_ERR_NO_DEVICE instead of falling back."""
    import ctypes
    import torch
    from mytrim_gb300 import _ffi as F
    lib = F.load()
    ctx = ctypes.c_void_p()
    st = lib.mtg_create(0, ctypes.byref(ctx))
    if torch.cuda.is_available():
        assert st == F.OK
        lib.mtg_destroy(ctx)
    else:
        assert st == 8  # MTG_ERR_NO_DEVICE
        assert not ctx.value
