"""C ABI: the library loads without a GPU and exports every symbol that a
header under include/ declares."""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    txt = "".join(p.read_text() for p in sorted((ROOT / "include").glob("*.h")))
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(edyn_[a-z_]+)\s*\(", txt)))


def test_header_declares_the_hot_path_entry_points():
    names = declared_functions()
    for n in ("edyn_init", "edyn_upload", "edyn_calc_dt", "edyn_solve_fluid", "edyn_solve_source", "edyn_post_step",
              "edyn_step", "edyn_advance", "edyn_download", "edyn_reactors", "edyn_last_error", "edyn_finalize"):
        assert n in names


def test_library_exports_every_declared_symbol():
    from fortrancfd_gb300 import lib

    L = lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing
    assert L.edyn_version().startswith(b"edyn-gb300")


def test_library_is_built_for_sm_103a_only():
    # the build passes exactly one -gencode for sm_103a
    src = (ROOT / "fortrancfd_gb300" / "build.py").read_text()
    assert 'ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]' in src


def test_product_path_does_not_touch_the_oracle():
    for p in (ROOT / "fortrancfd_gb300").rglob("*"):
        if p.suffix in (".py", ".cu", ".cpp", ".h", ".cuh") and p.name != "build.py":
            txt = p.read_text()
            for bad in ("oracle_ctypes", "libedyn_oracle", "edyn_oracle.h", "or_reactor", "or_step", "mlp_ref"):
                assert not re.search(r"\b" + re.escape(bad), txt), (p, bad)


def test_surrogate_constants_match_the_header():
    from fortrancfd_gb300 import surrogate as S

    txt = (ROOT / "include" / "edyn_surrogate.h").read_text()
    defs = dict(re.findall(r"#define (EDYN_MLP_EPI_\w+) (\d+)", txt))
    assert int(defs["EDYN_MLP_EPI_F32"]) == S.EPI_F32
    assert int(defs["EDYN_MLP_EPI_GELU"]) == S.EPI_GELU
    assert int(defs["EDYN_MLP_EPI_DGELU"]) == S.EPI_DGELU
    # padded widths are multiples of the GEMM's 64-column tiles
    assert S.KIN % 64 == 0 and S.KOUT % 64 == 0 and S.HID % 64 == 0
    assert S.NIN <= S.KIN and S.NOUT <= S.KOUT
