"""The C-ABI library without a GPU: it builds, loads, exports every symbol the
header declares, and its host-only entry points (tables, mesh) agree with the
reference's outputs."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "sipg_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sipg_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def built_lib():
    import sipg_gb300

    if not os.path.exists(sipg_gb300.LIB_PATH):
        import importlib.util

        spec = importlib.util.spec_from_file_location("sipg_build", os.path.join(ROOT, "cuda-sipg-matrix-free_gb300",
                                                                               "build.py"))
        m = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(m)
        m.build()
    return sipg_gb300


def test_header_compiles_as_c(tmp_path):
    src = tmp_path / "h.c"
    src.write_text('#include "sipg_gb300.h"\nint main(void){return (int)SIPG_OK;}\n')
    subprocess.check_call(["gcc", "-std=c99", "-Wall", "-Werror", "-fsyntax-only", "-I", os.path.join(ROOT, "include"),
                           str(src)])


def test_exports_every_declared_symbol(built_lib):
    L = built_lib.lib()
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_host_tables_match_reference(built_lib, golden):
    for n in range(2, 34):
        x, w = built_lib.lgl_table(n)
        np.testing.assert_allclose(x, golden["lgl_nodes_%d" % n], rtol=0, atol=4e-16)
        np.testing.assert_allclose(w, golden["lgl_weights_%d" % n], rtol=2e-14, atol=0)
    for p in range(1, 17):
        D = built_lib.dphi_table(p)
        ref = golden["dphi_%d" % p]
        assert np.max(np.abs(D - ref)) <= 2e-14 * np.max(np.abs(ref)), p


def _rows_from_laplace2d(L, p):
    """The mode_matrix rows of host_laplacian_matrix (mode_matrix.hpp:428-463)
    from the reference's laplace_2d values L[i1, i2, j1, j2]."""
    n = p + 1
    L = L.reshape(n, n, n, n)
    rows = []
    for i1 in range(n):
        for i2 in range(n):
            rows.append(L[i1, i2, i1, i2])
            rows += [L[i1, i2, i1, j] for j in range(n) if j != i2]
            rows += [L[i1, i2, j, i2] for j in range(n) if j != i1]
    return np.array(rows)


def test_laplacian_rows_match_reference(built_lib, golden):
    # the stored element Laplacian against the reference's own laplace_2d
    # values (tests/golden, from its code)
    for p in range(1, 9):
        rows = built_lib.laplacian_rows(p)
        ref = _rows_from_laplace2d(golden["laplace2d_%d" % p], p)
        assert rows.shape == ref.shape
        assert np.max(np.abs(rows - ref)) <= 1e-13 * np.max(np.abs(ref)), p


def test_mesh_coords_match_reference(built_lib, golden):
    for d in (1, 2, 3, 16):
        x, y = built_lib.square_mesh_coords(d)
        assert np.array_equal(x, golden["mesh_x_%d" % d])
        assert np.array_equal(y, golden["mesh_y_%d" % d])


def test_invalid_arguments_are_errors_not_crashes(built_lib):
    L = built_lib.lib()
    assert L.sipg_lgl_table(1, None, None) == 1
    assert L.sipg_dphi_table(64, None) == 1
    h = C.c_void_p()
    assert L.sipg_op_create(0, 4, 1.0, C.byref(h)) == 1
    assert L.sipg_op_create(4, 9, 1.0, C.byref(h)) == 5
    assert b"degree" in L.sipg_last_error()
    assert L.sipg_op_destroy(None) == 0
    assert L.sipg_op_solve_footprint(1024, 4, 0) > 6 * 26214400 * 8 - 1


@pytest.mark.parametrize("std,defines", [("c++14", []), ("c++14", ["-DUSE_PRECONDITIONER"]),
                                         ("c++14", ["-DUSE_MODE_MATRIX"]), ("c++17", [])])
def test_host_api_compiles_with_the_reference_flags(tmp_path, std, defines):
    # the reference's drivers build as C++14 with these switches; the host API
    # headers over the C ABI must accept the same (compile only: no GPU here)
    drv = os.path.join(ROOT, "tests", "cpp",
                       "host_api_pcg_driver.cpp" if "-DUSE_PRECONDITIONER" in defines else "host_api_driver.cpp")
    subprocess.check_call(["nvcc", "-std=" + std, "-O0", *defines, "-I", os.path.join(ROOT, "include"), "-I",
                           os.path.join(ROOT, "cuda-sipg-matrix-free_gb300", "host"), "-c", drv, "-o",
                           str(tmp_path / "drv.o")])


def test_integration_binding_example_compiles(tmp_path):
    # INTEGRATION.md's reference-side abs_mvm over the C ABI, against the host
    # headers with the reference's class names (compile only)
    subprocess.check_call(["nvcc", "-std=c++14", "-O0", "-I", os.path.join(ROOT, "include"), "-I",
                           os.path.join(ROOT, "cuda-sipg-matrix-free_gb300", "host"), "-c",
                           os.path.join(ROOT, "tests", "cpp", "integration_binding.cpp"), "-o",
                           str(tmp_path / "binding.o")])


def test_reference_style_kernel_compiles_against_mode_vector(tmp_path):
    # a device kernel indexing mode_vector as the reference's kernels do,
    # v(i1, i2, e) and get_noe() on the device (compile only: no GPU here)
    subprocess.check_call(["nvcc", "-std=c++14", "-O0", "-gencode", "arch=compute_103a,code=sm_103a", "-I",
                           os.path.join(ROOT, "include"), "-I",
                           os.path.join(ROOT, "cuda-sipg-matrix-free_gb300", "host"), "-c",
                           os.path.join(ROOT, "tests", "cpp", "mode_vector_kernel.cu"), "-o",
                           str(tmp_path / "mvk.o")])
