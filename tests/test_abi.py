"""Host-side checks of the C ABI that need no GPU: the library loads, exports every function
include/mbcg.h declares, and the Python mirrors of the structs match the C layout."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

import mbcg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "mbcg.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(mbcg_[a-z_0-9]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("mbcg_create", "mbcg_step", "mbcg_rcs_moments", "mbcg_bc_moments", "mbcg_copy_out",
                 "mbcg_diagnostics", "mbcg_destroy"):
        assert must in names


@pytest.mark.skipif(not os.path.exists(mbcg.LIB_PATH), reason="libmbcg.so not built")
def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(mbcg.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def _c_layout(struct, fields):
    src = "#include <stdio.h>\n#include <stddef.h>\n#include \"mbcg.h\"\nint main(void){\n"
    src += f'printf("%zu\\n", sizeof({struct}));\n'
    for f in fields:
        src += f'printf("%zu\\n", offsetof({struct}, {f}));\n'
    src += "return 0;}\n"
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    return [int(v) for v in out]


@pytest.mark.parametrize("pyt,cname", [(mbcg.Params, "mbcg_params"), (mbcg.Moments, "mbcg_moments"),
                                       (mbcg.Diag, "mbcg_diag"), (mbcg.ServerConfig, "mbcg_server_config"),
                                       (mbcg.RequestInfo, "mbcg_request_info"),
                                       (mbcg.ServerStats, "mbcg_server_stats"),
                                       (mbcg.PhaseStats, "mbcg_phase_stats")])
def test_struct_layout_matches_c(pyt, cname):
    names = [n for n, _ in pyt._fields_]
    c = _c_layout(cname, names)
    assert c[0] == ctypes.sizeof(pyt)
    for n, off in zip(names, c[1:]):
        assert getattr(pyt, n).offset == off, n


def test_presets_describe_the_benchmarked_cases():
    b = mbcg.bubble_params(64)
    assert (b.nx, b.ny, b.nz) == (66, 66, 66) and b.active_nodes() == 64 ** 3
    r = mbcg.rti_params(128)
    assert (r.nx, r.ny, r.nz) == (130, 130, 512) and r.bc[2] == mbcg.BC_WALL and r.rho_r0 == 3.0
    j = mbcg.jet_params()
    assert j.active_nodes() == 256 * 256 * 1024 and j.bc[2] == mbcg.BC_INOUT
    assert j.outlet == mbcg.OUTLET_ZERO_GRADIENT and abs(j.jet_radius - 16.0) < 1e-12


def test_noise_generator_is_uniform_and_seeded():
    import oracle_lib as ol
    xs = [ol.oracle_noise(12345, 7, n, c) for n in range(2000) for c in range(3)]
    assert min(xs) >= -1.0 and max(xs) < 1.0
    assert abs(sum(xs) / len(xs)) < 0.05
    assert ol.oracle_noise(12345, 7, 11, 0) == ol.oracle_noise(12345, 7, 11, 0)
    assert ol.oracle_noise(12345, 7, 11, 0) != ol.oracle_noise(12345, 8, 11, 0)


@pytest.mark.parametrize("field,value", [("max_live", 65), ("chunk_steps", 2000), ("zchunk", -1), ("policy", 7)])
def test_server_config_is_validated_before_any_device_work(field, value):
    """mbcg_server_create rejects a configuration outside its limits (at most 64 live lattices:
    the batch kernel's constant parameter table) with MBCG_E_INVALID, before touching a GPU."""
    lib = mbcg.Library.get()
    cfg = mbcg.ServerConfig()
    lib.mbcg_server_config_default(ctypes.byref(cfg))
    setattr(cfg, field, value)
    h = ctypes.c_void_p()
    assert lib.mbcg_server_create(ctypes.byref(cfg), ctypes.byref(h)) == -1  # MBCG_E_INVALID
    assert not h.value


def test_run_host_rejects_a_null_case():
    lib = mbcg.Library.get()
    assert lib.mbcg_run_host(None, 0, None, None, 1, None) == -1  # MBCG_E_INVALID
