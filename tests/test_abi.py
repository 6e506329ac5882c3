"""The C-ABI library loads and exports every function its headers declare
(CPU-only: no CUDA call is made)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = ["calCommon.h", "cal2D.h", "cal2DRun.h", "cal2DIO.h", "cal2DReduction.h", "cal2DUnsafe.h", "cal3D.h",
           "cal3DRun.h", "cal3DUnsafe.h",
           "cal3DIO.h", "cal3DReduction.h"]


def declared_functions(headers=HEADERS):
    names = set()
    for h in headers:
        text = open(os.path.join(ROOT, "include", "opencal", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = text.split("#if defined(__CUDACC__)")[0]  # device-side helpers are not exports
        for m in re.finditer(r"^[A-Za-z][\w\s\*]*?\b(cal\w+)\s*\(", text, flags=re.M):
            if not m.group(0).lstrip().startswith(("typedef", "#")):
                names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    import opencal_gb300 as cal
    cal.build()
    return cal.core()


def test_headers_declare_the_reference_api():
    names = set(declared_functions())
    for fn in ["calCADef2D", "calAddSubstate2Db", "calAddSubstate2Di", "calAddSubstate2Dr",
               "calAddElementaryProcess2D", "calRun2D", "calAddActiveCell2D", "calUpdateActiveCells2D",
               "calCADef3D", "calRun3D", "calGetX2Dr", "calSet2Dr", "calUpdate2D", "calRunCAStep2D"]:
        assert fn in names, fn
    assert len(names) > 150


def test_library_exports_every_declared_function(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_models_library_exports_every_declared_function():
    import opencal_gb300 as cal
    m = cal.models()
    names = declared_functions(["calModels.h"])
    for fn in ["cal_sciddicaT_run", "cal_sdt_adj_backward", "cal_sdt_batch_loss_grad", "cal_life2d_run"]:
        assert fn in names, fn
    missing = [n for n in names if not hasattr(m, n)]
    assert not missing, missing


def test_no_cpu_fallback_without_libs(tmp_path, monkeypatch):
    import opencal_gb300 as cal
    monkeypatch.setattr(cal, "CORE_LIB", str(tmp_path / "missing.so"))
    monkeypatch.setattr(cal, "_core", None)
    with pytest.raises(cal.CALError):
        cal.core()
