"""The C-ABI library builds, loads and exports every function include/lqg.h declares."""
import ctypes as C
import os
import re

import golden_cases  # noqa: F401  (puts the repo root on sys.path via conftest)
from lyspeq_gb300 import lqg

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "lqg.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_]+\s*\*?\s*(lqg_[a-z_0-9]+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "lqg_nr_iteration" in names and "lqg_batch_add" in names
    assert set(lqg.EXPORTS) <= set(names)


def test_library_exports_header(engine_lib):
    for name in declared_functions():
        assert hasattr(engine_lib, name), name


def test_null_arguments_rejected_without_gpu(engine_lib):
    h = C.c_void_p()
    assert engine_lib.lqg_ctx_create(C.byref(h), None, None, None, 0) == -1
    assert engine_lib.lqg_abi_version() == 3


def test_tuning_field_count_matches_the_header():
    text = open(HEADER).read()
    m = re.search(r"#define LQG_TUNING_FIELDS (\d+)", text)
    assert m and int(m.group(1)) == lqg.TUNING_FIELDS


def test_python_mirror_types_every_entry_point():
    """lyspeq_gb300/lqg.py declares the argument types of every function of
    include/lqg.h and lists it among the exports it checks."""
    import re
    from lyspeq_gb300 import lqg
    declared = set(re.findall(r"^(?:int|const char \*|double|void)\s*\*?\s*(lqg_[a-z_0-9]+)\s*\(",
                              open(HEADER).read(), re.M))
    typed = set(re.findall(r"lib\.(lqg_[a-z_0-9]+)\.argtypes", open(lqg.__file__).read()))
    assert declared and declared == typed
    assert declared == set(lqg.EXPORTS)
