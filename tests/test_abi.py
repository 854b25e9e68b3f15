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


def test_header_compiles_as_c99_and_cxx(tmp_path):
    """include/kcore.h is a plain C header (the boundary a cgo / JNI / ctypes
    host binds): it compiles on its own as C99 and as C++17, and a C++
    program that includes it links against libkcore.so and runs."""
    import shutil
    import subprocess
    from pico_gb300 import build as pb
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    inc = os.path.join(root, "include")
    c = tmp_path / "use.c"
    c.write_text('#include "kcore.h"\nint f(kc_graph *g) { kc_stats st; return kc_decompose(g, KC_PEELONE_DYN, '
                 '0, 0, &st, 0) + (int)st.kmax + KC_ABI_VERSION; }\n')
    for cc, std, src in (("gcc", "-std=c99", c), ("g++", "-std=c++17", c)):
        if shutil.which(cc) is None:
            continue
        args = [cc, std, "-Wall", "-Werror", "-fsyntax-only", "-I", inc]
        if cc == "g++":
            args += ["-x", "c++"]
        r = subprocess.run(args + [str(src)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
    lib = pb.LIB
    if shutil.which("g++") and os.path.exists(lib):
        cpp = tmp_path / "app.cpp"
        cpp.write_text('#include "kcore.h"\n#include <cstdio>\nint main() { std::printf("%d\\n", kc_abi_version()); '
                       'return 0; }\n')
        exe = tmp_path / "app"
        r = subprocess.run(["g++", "-I", inc, str(cpp), "-L", os.path.dirname(lib), "-lkcore",
                            "-Wl,-rpath," + os.path.dirname(lib), "-o", str(exe)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        r = subprocess.run([str(exe)], capture_output=True, text=True)
        assert r.returncode == 0 and r.stdout.strip() == "1", (r.stdout, r.stderr)
