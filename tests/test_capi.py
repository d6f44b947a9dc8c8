"""C ABI: exported symbols, option parsing and error behaviour (CPU only)."""
import ctypes
import os
import re
import subprocess

import pytest

import miniaero_gb300 as ma
from miniaero_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "miniaero_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ma_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "ma_mesh_upload" in names and "ma_solver_step" in names and len(names) > 30


def test_library_exports_every_declared_symbol():
    out = subprocess.check_output(["nm", "-D", "--defined-only", _lib.LIB_PATH], text=True)
    exported = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing


def test_abi_version_and_status_strings():
    L = _lib.lib()
    assert L.ma_abi_version() == 1
    assert L.ma_status_string(_lib.MA_EBUDGET) == b"over device-memory budget"


def write(tmp_path, text):
    p = tmp_path / "miniaero.inp"
    p.write_text(text)
    return str(p)


def test_read_reference_inputs(reference_dir):
    for case, expect in [("3D_Sod_Serial", (0, 128, 4, 4, 100, 2e-6, 0, 0)),
                         ("Ramp_Serial", (2, 64, 32, 2, 400, 1e-5, 1, 0)),
                         ("FlatPlate_Serial", (1, 16, 32, 2, 400, 3e-8, 1, 1))]:
        o = ma.Options.read_options_file(os.path.join(reference_dir, "tests", case, "miniaero.inp"))
        got = (o.problem_type, o.nx, o.ny, o.nz, o.ntimesteps, o.dt, o.second_order_space, o.viscous)
        assert got == expect


def test_extension_keys(tmp_path):
    path = write(tmp_path, "1\n2.0 0.5 0.5 0.0\n64 16 16\n50\n1e-6\n1\n10\n1\n1\n"
                           "limiter vanalbada\nviscosity constant 1.8e-5 0.72\nprecision mixed\ncfl 0.5\n"
                           "sod 1 1 0.125 0.1\n# comment line\ninflow 1.2 100 0 0 250000\nbc bottom noslip\n"
                           "keep_residual 1\n")
    o = ma.Options.read_options_file(path)
    assert o.limiter == ma.MA_LIMITER_VANALBADA
    assert o.viscosity_model == ma.MA_VISC_CONSTANT and o.mu == 1.8e-5 and o.prandtl == 0.72
    assert o.precision == ma.MA_PREC_MIXED and o.cfl == 0.5
    assert o.ic == ma.MA_IC_SOD and o.sod_right == [0.125, 0.1]
    assert o.inflow_state == [1.2, 100.0, 0.0, 0.0, 250000.0]
    assert o.bc_override[0] == ma.MA_BC_NOSLIP and o.keep_residual == 1


def test_precision_keys(tmp_path):
    base = "0\n1 1 1 0\n4 4 4\n10\n1e-5\n0\n1\n0\n0\n"
    for word, want in (("fp64", ma.MA_PREC_FP64), ("mixed", ma.MA_PREC_MIXED), ("fp64_fma", ma.MA_PREC_FP64_FMA)):
        o = ma.Options.read_options_file(write(tmp_path, base + "precision %s\n" % word))
        assert o.precision == want
    with pytest.raises(ma.MiniaeroError):
        ma.Options.read_options_file(write(tmp_path, base + "precision fp16\n"))


@pytest.mark.parametrize("text", ["0\n1 1 1 0\n4 4\n", "0\n1 1 1 0\n4 4 4\n10\n1e-5\n0\n1\n0\n0\nbogus 3\n",
                                  "0\n1 1 1 0\n4 4 4\n10\n1e-5\n0\n1\n0\n0\nlimiter minmod\n"])
def test_malformed_inputs_are_errors(tmp_path, text):
    with pytest.raises(ma.MiniaeroError) as e:
        ma.Options.read_options_file(write(tmp_path, text))
    assert e.value.status == _lib.MA_EINVAL


def test_missing_input_is_io_error(tmp_path):
    with pytest.raises(ma.MiniaeroError) as e:
        ma.Options.read_options_file(str(tmp_path / "nope.inp"))
    assert e.value.status == _lib.MA_EIO


def test_defaults_match_reference_constructor():
    o = ma.Options()
    assert (o.problem_type, o.nx, o.ny, o.nz, o.ntimesteps, o.dt, o.output_frequency) == (0, 10, 10, 10, 1, 5e-8, 10)
    assert o.inflow_state == [0.5805, 503.96, 0.0, 0.0, 343750.0]


def test_device_calls_fail_cleanly_without_gpu():
    if ma.device_count() > 0:
        pytest.skip("a GPU is present")
    o = ma.Options(nx=4, ny=2, nz=2)
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    with pytest.raises(ma.MiniaeroError) as e:
        ma.TimeSolverExplicitRK4(md, o)
    assert e.value.status == _lib.MA_ECUDA
    with pytest.raises(ma.MiniaeroError):
        ma.roe_flux([[1, 0, 0, 0, 300]], [[1, 0, 0, 0, 300]], [[1, 0, 0]], [[0, 1, 0]], [[0, 0, 1]])
    with pytest.raises(ma.MiniaeroError):
        ma.fp64_rate("add")


def test_upload_rejects_bad_meshes():
    o = ma.Options(nx=3, ny=2, nz=2)
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    md.internal.permutation[0] = md.internal.permutation[1]
    with pytest.raises(ma.MiniaeroError) as e:
        ma.DeviceMesh(md)
    assert e.value.status == _lib.MA_EINVAL
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    md.internal.conn[0, 1] = md.ncells + 5
    with pytest.raises(ma.MiniaeroError) as e:
        ma.DeviceMesh(md)
    assert e.value.status == _lib.MA_EINVAL
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    md.cell_volumes[2] = -1.0
    with pytest.raises(ma.MiniaeroError) as e:
        ma.DeviceMesh(md)
    assert e.value.status == _lib.MA_EINVAL


def test_upload_rejects_meshes_beyond_32bit_indexing():
    """The gradient arrays are indexed (3k + d) C + c in 32-bit arithmetic:
    meshes above MA_MAX_MESH_CELLS are refused before any array is read."""
    assert 15 * 143165576 <= 2 ** 31 - 1 < 15 * 143165577
    view = _lib.ma_mesh_view()
    view.ncells = 143165577
    h = ctypes.c_void_p()
    st = _lib.lib().ma_mesh_upload_ex(ctypes.byref(view), 0, ctypes.byref(h))
    assert st == _lib.MA_EINVAL and not h
    assert b"143165576" in _lib.lib().ma_last_error()
    # The host mesh generator refuses such a box before building it.
    with pytest.raises(ma.MiniaeroError) as e:
        ma.Parallel3DMesh.from_options(ma.Options(nx=524, ny=524, nz=524)).fill_mesh_data()
    assert e.value.status == _lib.MA_EINVAL


def test_cli_reports_missing_input(tmp_path):
    from miniaero_gb300 import build as b
    r = subprocess.run([b.CLI], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode != 0
    assert "does not exist" in r.stderr


def declared_prototypes():
    """{name: (return type text, [parameter texts])} from the header."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"#.*", "", text)
    protos = {}
    for m in re.finditer(r"([A-Za-z_][A-Za-z0-9_ \*]*?)\s*\b(ma_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", text, flags=re.S):
        ret, name, params = m.group(1).strip(), m.group(2), " ".join(m.group(3).split())
        args = [] if params in ("", "void") else [p.strip() for p in params.split(",")]
        protos[name] = (ret, args)
    return protos


def test_ctypes_signatures_match_the_header():
    """Every declared entry point has a ctypes signature with the header's
    argument count, pointer parameters as pointers and the right return kind."""
    protos = declared_prototypes()
    assert set(protos) == set(declared_functions())
    sigs = _lib._SIGNATURES
    missing = sorted(set(protos) - set(sigs))
    assert not missing, missing
    for name, (ret, args) in protos.items():
        res, argtypes = sigs[name]
        assert len(argtypes) == len(args), (name, args, argtypes)
        for text, t in zip(args, argtypes):
            is_ptr = "*" in text
            ctypes_ptr = t in (ctypes.c_void_p, ctypes.c_char_p) or (isinstance(t, type) and issubclass(
                t, (ctypes._Pointer,)))
            assert is_ptr == ctypes_ptr, (name, text, t)
        if ret == "void":
            assert res is None, name
        elif "*" in ret:
            assert res in (ctypes.c_void_p, ctypes.c_char_p), (name, ret, res)
        else:
            assert res is not None, name


def test_header_is_plain_c(tmp_path):
    """The boundary is a C ABI: the header compiles as strict C99 and a C
    program links against the library and calls it (no GPU needed)."""
    from miniaero_gb300 import build as b
    src = tmp_path / "main.c"
    src.write_text('#include <stdio.h>\n#include "miniaero_gpu.h"\n'
                   "int main(void) { ma_options o; ma_options_default(&o);\n"
                   '  printf("%d %d %s\\n", ma_abi_version(), o.nx, ma_status_string(MA_EINVAL)); return 0; }\n')
    exe = tmp_path / "main"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.dirname(HEADER),
                    str(src), "-L", b.BUILD, "-lminiaero_gpu", "-Wl,-rpath," + b.BUILD, "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert out[0] == "1" and out[1] == "10"
