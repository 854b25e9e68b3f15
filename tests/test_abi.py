"""The C-ABI library loads and exports every symbol include/kcore.h declares
(no compute calls: this runs without a GPU)."""
import ctypes
import os

import pico_gb300 as pg


def test_library_exports_every_declared_symbol():
    L = pg.lib()
    names = pg.header_symbols()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert missing == []


def test_abi_version_and_error_string():
    assert pg.lib().kc_abi_version() == 1
    assert isinstance(pg.lib().kc_last_error(), bytes)


def test_no_gpu_fails_loudly_not_silently():
    if pg.device_count() > 0:
        return  # with a GPU present this path is covered by the gpu tests
    try:
        pg.Graph.from_edges([0, 1], [1, 2], 3)
    except pg.KCoreError as e:
        assert e.code == pg.KC_ERR_CUDA
    else:
        raise AssertionError("graph build without a GPU must fail")


def test_cli_drivers_built():
    from pico_gb300 import build as pb
    for name in ("HistoCore", "CntCore", "NbrCore", "peelone", "gppeel", "peelone_dyn"):
        p = os.path.join(pb.BIN, name)
        if os.path.exists(os.path.join(pb.CLI, name + ".cpp")):
            assert os.access(p, os.X_OK), p
