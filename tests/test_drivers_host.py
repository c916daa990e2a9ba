"""Host-side behaviour of the drop-in driver executables that needs no GPU:
argument and input-file errors, popfile-list errors, and -- on a machine
without a GPU -- a clean failure at context creation after all files were
read (no CPU fallback)."""
import subprocess

import pytest

from driver_util import BUILD, stage_pops_run


@pytest.fixture(scope="module")
def drivers(clbm_lib):
    import build as b
    b.build_drivers()
    return BUILD


def run(exe, args, cwd):
    return subprocess.run([str(exe), *args], cwd=cwd, capture_output=True, text=True, timeout=120)


def test_usage_without_input(drivers, tmp_path):
    r = run(drivers / "TLGK_LBM_POPS_PERTURB", [], tmp_path)
    assert r.returncode == 2 and "usage" in r.stderr


def test_missing_input_file(drivers, tmp_path):
    r = run(drivers / "TLGK_LBM_POPS_PERTURB", ["nope"], tmp_path)
    assert r.returncode == 1
    assert "COULD NOT OPEN INPUT FILE" in (tmp_path / "output_TLGK.out").read_text()


def test_missing_popfile_list(drivers, tmp_path, orc):
    stage_pops_run(orc, tmp_path, dict(L=4, Nc=4, U0=0.05, tau=0.6, alpha=1.0, eps=0.01, T=1.0, dT=0.25))
    (tmp_path / "pops" / "popfiles_list.dat").unlink()
    r = run(drivers / "TLGK_LBM_POPS_PERTURB", ["input"], tmp_path)
    assert r.returncode == 1
    assert "COULD NOT OPEN INDEX FILE" in (tmp_path / "output_TLGK.out").read_text()


def test_ranks_must_divide(drivers, tmp_path, orc):
    stage_pops_run(orc, tmp_path, dict(L=4, Nc=4, U0=0.05, tau=0.6, alpha=1.0, eps=0.01, T=1.0, dT=0.25))
    r = run(drivers / "TLGK_LBM_POPS_PERTURB", ["--ranks", "3", "input"], tmp_path)
    assert r.returncode == 1
    assert "multiple of --ranks" in (tmp_path / "output_TLGK.out").read_text()


def test_no_gpu_fails_cleanly_after_reading_inputs(drivers, tmp_path, orc, clbm_lib):
    if clbm_lib.device_count() > 0:
        pytest.skip("a GPU is present")
    stage_pops_run(orc, tmp_path, dict(L=4, Nc=4, U0=0.05, tau=0.6, alpha=1.0, eps=0.01, T=1.0, dT=0.25))
    r = run(drivers / "TLGK_LBM_POPS_PERTURB", ["input"], tmp_path)
    assert r.returncode == 1
    log = (tmp_path / "output_TLGK.out").read_text()
    assert "Dx = 17" in log and "no CUDA device" in log
    assert (tmp_path / "out" / "clone_3").is_dir()
