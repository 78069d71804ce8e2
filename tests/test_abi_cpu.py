"""C-ABI library checks that need no GPU: it builds for sm_103a, loads, exports
every entry point declared in include/ice3gb.h and rejects bad arguments
before touching the device."""
import ctypes
import os
import re

import pytest

from conftest import REPO


@pytest.fixture(scope="module")
def lib():
    import importlib.util
    spec = importlib.util.spec_from_file_location("ice3gb_build", os.path.join(REPO, "dwarf-p-ice3_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()
    from ice3gb import _abi
    return _abi.load()


def declared_functions():
    text = open(os.path.join(REPO, "include", "ice3gb.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int64_t|int|const char \*)\s*(ice3gb_\w+)\(", text, re.M)))


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 14
    for n in names:
        assert hasattr(lib, n), n
    from ice3gb import _abi
    assert set(_abi.EXPORTED) == set(names)


def test_constant_names_match_header(lib):
    from ice3gb.constants import CONSTANT_NAMES
    n = lib.ice3gb_constant_count()
    assert n == len(CONSTANT_NAMES)
    assert [lib.ice3gb_constant_name(i).decode() for i in range(n)] == CONSTANT_NAMES
    assert lib.ice3gb_constant_name(n) is None
    assert lib.ice3gb_version() == 10000


def test_rejects_null_and_bad_handle(lib):
    from ice3gb import _abi
    h = ctypes.c_void_p()
    assert lib.ice3gb_create(None, None, ctypes.byref(h)) == -1
    bogus = ctypes.c_void_p(0x1000)
    f = _abi.IceAdjustFields()
    assert lib.ice3gb_ice_adjust(None, 4, 4, 50.0, ctypes.byref(f), None) == -7
    assert lib.ice3gb_rain_ice(None, 4, 4, 50.0, None, None, None) == -7
    assert lib.ice3gb_physics_step(None, 4, 4, 50.0, None, None, None) == -7
    buf = ctypes.create_string_buffer(256)
    assert lib.ice3gb_last_error(None, buf, 256) > 0
    assert b"invalid handle" in buf.value
    assert lib.ice3gb_destroy(None) == -7
    del bogus
