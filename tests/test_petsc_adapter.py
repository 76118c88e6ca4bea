"""The PETSc adapter (include/sbp_petsc.h, hpc-reading-course_gb300/petsc/sbp_petsc.cpp), built
against a minimal stand-in of the PETSc calls it makes (tests/petsc_shim/) and linked with
libsbpgpu: the RHS callback the reference registers with TSSetRHSFunction
(code/src/time_stepping/ts_rk.cpp:21) and the ts_rk4 / ts_rk45 drop-ins (ts_rk.cpp:41-65).

CPU: it compiles, and null contexts come back as PETSC_ERR_ARG_NULL with no array left
checked out. GPU: the adapter gives the bits of sbp_rhs and sbp_ts_rk4, a vector of the wrong
size is PETSC_ERR_ARG_SIZ, a failing library call PETSC_ERR_LIB naming the call."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "tests", "petsc_shim")


def _build(sbp, tmp_path):
    import build as gpu_build

    lib_dir = os.path.dirname(gpu_build.LIB)
    shim_o = str(tmp_path / "petsc_shim.o")
    exe = str(tmp_path / "adapter_check")
    subprocess.run(["gcc", "-std=c11", "-O1", "-c", os.path.join(SHIM, "petsc_shim.c"), "-I", SHIM, "-o", shim_o],
                   check=True)
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I", SHIM, "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "hpc-reading-course_gb300", "petsc", "sbp_petsc.cpp"),
                    os.path.join(SHIM, "adapter_check.cpp"), shim_o, "-L", lib_dir, "-lsbpgpu",
                    "-Wl,-rpath," + lib_dir, "-o", exe], check=True)
    return exe


def test_adapter_builds_and_rejects_null_contexts(sbp, tmp_path):
    exe = _build(sbp, tmp_path)
    r = subprocess.run([exe, "cpu"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "FAIL" not in r.stdout and r.stdout.count("ok") == 4


@pytest.mark.gpu
def test_adapter_matches_the_library_on_a_device(sbp, tmp_path):
    exe = _build(sbp, tmp_path)
    r = subprocess.run([exe, "gpu"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "FAIL" not in r.stdout and "rhs: the same bits" in r.stdout and "ts_rk4: the same bits" in r.stdout


def test_adapter_build_looks_for_petsc_headers(tmp_path, monkeypatch):
    """build_petsc_adapter() builds only where $PETSC_DIR[/$PETSC_ARCH] holds petscts.h."""
    import build as gpu_build

    monkeypatch.delenv("PETSC_DIR", raising=False)
    assert gpu_build.petsc_include_dirs() is None
    assert gpu_build.build_petsc_adapter() is None
    monkeypatch.setenv("PETSC_DIR", str(tmp_path))
    monkeypatch.setenv("PETSC_ARCH", "arch-test")
    assert gpu_build.petsc_include_dirs() is None  # no headers there
    (tmp_path / "include").mkdir()
    (tmp_path / "include" / "petscts.h").write_text("/* stand-in */\n")
    assert gpu_build.petsc_include_dirs() == [str(tmp_path / "include"), str(tmp_path / "arch-test" / "include")]
