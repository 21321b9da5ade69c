"""CPU checks of the C-ABI library: it builds, loads without a GPU, exports
every function include/hosnwt.h declares, and its host-only parser reads the
reference's input format."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    txt = open(os.path.join(ROOT, "include", "hosnwt.h")).read()
    return sorted(set(re.findall(r"\b(hosnwt_[A-Za-z0-9_]+)\s*\(", txt)))


def test_library_exports_header(lib):
    import hosnwt
    names = _declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    assert set(hosnwt.C_FUNCTIONS) <= set(names)


def test_read_input_host_only(lib):
    import hosnwt
    d = hosnwt.read_input(os.path.join(ROOT, "tests", "golden", "input_HOS-NWT.dat"))
    assert d["xlen"] == 50.0 and d["ylen"] == 30.0 and d["h"] == 5.0
    assert d["icase"] == 2 and d["ibat"] == 2 and d["i_wmk"] == 1 and d["igeom"] == 2
    assert d["file_name"] == "J010_14" and d["pro_file"] == "prob.inp"
    assert d["toler"] == 1e-7 and d["f_out"] == 10.0 and d["Tramp"] == 3.0


def test_read_input_matches_oracle_parser(lib):
    import hosnwt
    from oracle.hos_oracle import read_input
    p = os.path.join(ROOT, "tests", "golden", "input_HOS-NWT.dat")
    a, b = hosnwt.read_input(p), read_input(p)
    for k, v in b.items():
        assert a[k] == v, k


def test_missing_input_is_an_error(lib):
    import hosnwt
    with pytest.raises(RuntimeError):
        hosnwt.read_input("/nonexistent/input_HOS-NWT.dat")


def test_noalloc_limit_matches_header():
    import hosnwt
    txt = open(os.path.join(ROOT, "include", "hosnwt.h")).read()
    m = re.search(r"#define\s+HOSNWT_NOALLOC_MAX_N\s+(\d+)", txt)
    assert m and int(m.group(1)) == hosnwt.NOALLOC_MAX_N
