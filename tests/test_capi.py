"""The C ABI library builds, loads and exports every symbol its header declares;
argument checks that need no device behave like the upstream class (CPU only)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "hpdbscan_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hpd_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_the_abi():
    names = declared_functions()
    for required in ("hpd_create", "hpd_destroy", "hpd_cluster", "hpd_cluster_device", "hpd_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol(engine_lib):
    for name in declared_functions():
        assert hasattr(engine_lib, name), name


def test_python_binding_lists_the_exports(engine_lib):
    from hpdbscan_gb300 import _lib
    for name in _lib.EXPORTS:
        assert hasattr(engine_lib, name)
    assert set(_lib.EXPORTS) <= set(declared_functions())


@pytest.mark.parametrize("eps", [0.0, -1.0, float("nan")])
def test_create_rejects_bad_epsilon(engine_lib, eps):
    h = ctypes.c_void_p()
    rc = engine_lib.hpd_create(eps, 5, ctypes.byref(h))
    assert rc == 1
    assert engine_lib.hpd_last_error() == b"epsilon needs to be positive"
    assert not h.value


def test_python_class_raises_value_error(engine_lib):
    from hpdbscan_gb300 import HPDBSCAN
    with pytest.raises(ValueError, match="epsilon needs to be positive"):
        HPDBSCAN(-0.5, 3)


def test_cluster_rejects_null_handle(engine_lib):
    rc = engine_lib.hpd_cluster(None, None, 0, 2, 0, 1, None)
    assert rc == 1


def test_version_string(engine_lib):
    assert engine_lib.hpd_version().startswith(b"hpdbscan_gb300")


def test_tuning_table_bounds(engine_lib):
    from hpdbscan_gb300 import _lib
    arr = (_lib.TuningEntry * 65)()
    assert engine_lib.hpd_set_tuning_table(arr, 65) == 1
    assert engine_lib.hpd_set_tuning_table(None, 1) == 1
    assert engine_lib.hpd_set_tuning_table(None, 0) == 0
