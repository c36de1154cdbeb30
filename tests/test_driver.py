"""sphnj_run, the host driver: command line and failure behaviour (CPU)."""
from __future__ import annotations

import subprocess

import pytest
import torch

import sphnj_gb300 as S
from sphnj_gb300 import _build, cases


@pytest.fixture(scope="module")
def driver():
    S.build()
    assert _build.DRIVER.exists()
    return str(_build.DRIVER)


def test_help(driver):
    r = subprocess.run([driver, "--help"], capture_output=True, text=True)
    assert r.returncode == 0
    assert "usage: sphnj_run CASE_DIR" in r.stdout


@pytest.mark.parametrize("argv", [[], ["--form", "double"], ["x", "--global", "nope"], ["x", "--probe", "1"],
                                  ["x", "y"], ["x", "--iend"]])
def test_bad_command_lines(driver, argv):
    r = subprocess.run([driver, *argv], capture_output=True, text=True)
    assert r.returncode == 2, r.stderr


def test_missing_case(driver, tmp_path):
    r = subprocess.run([driver, str(tmp_path / "none")], capture_output=True, text=True)
    assert r.returncode == 1
    assert "input.ini" in r.stderr


def test_incomplete_ini_is_refused(driver, tmp_path):
    case = cases.dam_break_water(dx=0.1, iend=5)
    del case.ini["dt"]  # a key readParameter requires (sim_time.cpp:10-16)
    case.write(tmp_path / "c")
    r = subprocess.run([driver, str(tmp_path / "c")], capture_output=True, text=True)
    assert r.returncode == 1
    assert "required key" in r.stderr


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the no-device path")
def test_no_device_is_reported(driver, tmp_path):
    cases.dam_break_water(dx=0.1, iend=5).write(tmp_path / "c")
    r = subprocess.run([driver, str(tmp_path / "c")], capture_output=True, text=True)
    assert r.returncode == 3
    assert "status 11" in r.stderr
