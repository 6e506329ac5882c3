"""The SCIARA-fv2 configuration reader (cal_sciara_read, host code of
libopencal_models.so; no GPU needed) on the reference's shipped 2006 files
(stored byte for byte in tests/golden/sciara_2006.npz): the values it
returns are those the files hold, read the reference's way (io.cpp,
GISInfo.cpp, vent.cpp of the SCIARA-fv2 example), and malformed files are
refused with CAL_ERROR_IO."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = {"file_000000000000_cfg": "2006_000000000000.cfg", "file_Morphology_stt": "2006_000000000000_Morphology.stt",
         "file_Vents_stt": "2006_000000000000_Vents.stt", "file_EmissionRate_txt": "2006_000000000000_EmissionRate.txt"}


def _write(tmp_path):
    fx = np.load(os.path.join(GOLDEN, "sciara_2006.npz"))
    for key, name in NAMES.items():
        (tmp_path / name).write_bytes(fx[key].tobytes())
    return fx


def _grid(text):
    tok = text.split()
    head = dict(zip(tok[0:12:2], tok[1:12:2]))
    rows, cols = int(head["nrows"]), int(head["ncols"])
    return np.array([float(x) for x in tok[12:]]).reshape(rows, cols), float(head["cellsize"])


def test_reader_returns_the_files_values(tmp_path):
    import opencal_gb300 as cal
    _write(tmp_path)
    c = cal.sciara_read(str(tmp_path / "2006"))
    z, cell = _grid((tmp_path / NAMES["file_Morphology_stt"]).read_text())
    assert c["z"].tobytes() == z.tobytes()
    mv, _ = _grid((tmp_path / NAMES["file_Vents_stt"]).read_text())
    want = [(int(k % mv.shape[1]), int(k // mv.shape[1])) for k in np.flatnonzero(mv.ravel() > 0)]
    assert [tuple(int(a) for a in v) for v in c["vents"]] == want
    cfg = (tmp_path / NAMES["file_000000000000_cfg"]).read_text().split()
    vals = dict(zip(cfg[0::2], cfg[1::2]))
    keys = ["Pclock", "PTsol", "PTvent", "Pr(Tsol)", "Pr(Tvent)", "Phc(Tsol)", "Phc(Tvent)", "Pcool", "Prho",
            "Pepsilon", "Psigma", "Pcv"]
    assert list(c["params"]) == [float(vals[k]) for k in keys] + [cell]
    em = (tmp_path / NAMES["file_EmissionRate_txt"]).read_text().split()
    assert c["emission_time"] == int(em[1])
    first = em.index("[EMISSION_RATE]")
    stop = em.index("[VENT_ID]", first)
    assert c["rates"][0] == [float(x) for x in em[first + 1:stop]]
    # the path may also name the .cfg itself
    c2 = cal.sciara_read(str(tmp_path / NAMES["file_000000000000_cfg"]))
    assert c2["z"].tobytes() == c["z"].tobytes()


def test_reader_refuses_malformed_files(tmp_path):
    import opencal_gb300 as cal
    _write(tmp_path)
    morph = tmp_path / NAMES["file_Morphology_stt"]
    text = morph.read_text()
    morph.write_text(text.rsplit(" ", 3)[0])  # values missing at the end
    with pytest.raises(cal.CALError):
        cal.sciara_read(str(tmp_path / "2006"))
    morph.write_text(text)
    (tmp_path / NAMES["file_EmissionRate_txt"]).write_text("[TIME]\n86400\n\n[VENT_ID]\n9\n[EMISSION_RATE]\n1\n[END]\n")
    with pytest.raises(cal.CALError):
        cal.sciara_read(str(tmp_path / "2006"))  # vent 9 is not on the grid, vents 1 and 2 have no rates
