"""The `vecsz` command line (vecsz_gb300/cli/vecsz_cli.cpp): the reference's flags and checks
(src/argument_parser/argparse.cc).  These cases stop in argument checking, before any GPU call."""
import os
import subprocess

import pytest

import vecsz_gb300 as V
from vecsz_gb300 import _build

CLI = _build.CLI


@pytest.fixture(scope="module")
def cli():
    V.lib()  # builds the library and the command line if needed
    assert os.path.exists(CLI)
    return CLI


def run(cli, *args):
    return subprocess.run([cli, *args], capture_output=True, text=True, timeout=60)


def test_cli_version_and_help(cli):
    r = run(cli, "-v")
    assert r.returncode == 0 and "sm_103a" in r.stdout
    r = run(cli, "--help")
    assert r.returncode == 0 and "--compress" in r.stdout and "-L, --lossless" in r.stdout
    r = run(cli)
    assert r.returncode == 0 and "dry-run" in r.stdout


def test_cli_argument_errors(cli):
    r = run(cli, "-z", "-i", "field.f32")
    assert r.returncode == 255
    assert "Incorrect input size(s)!" in r.stderr and "Not specifying data type!" in r.stderr
    r = run(cli, "-z", "-t", "f32", "-l", "8,8,8")
    assert r.returncode == 255 and "Not specifying input file!" in r.stderr
    r = run(cli, "-t", "f32", "-l", "8,8,8", "-i", "f")
    assert r.returncode == 255 and "Select compress (-z), decompress (-x), or dry-run (-r)!" in r.stderr
    r = run(cli, "-q")
    assert r.returncode == 255 and "invalid option value at position 1" in r.stderr
    r = run(cli, "-z", "-t", "f32", "-l", "8,x", "-i", "f")
    assert r.returncode == 255 and "non-convertible part: x" in r.stderr
    r = run(cli, "-z", "-t", "f32", "-l", "8,8,8", "-i", "f", "--num-iter", "3")
    assert r.returncode == 255 and "Autotune option not specified!" in r.stderr
    r = run(cli, "-z", "-t", "f32", "-l", "8,8,8,2", "-i", "f")
    assert r.returncode == 255 and "4D fields" in r.stderr
    r = run(cli, "-z", "-t", "f32", "-D", "nowhere", "-i", "f")
    assert r.returncode == 255 and "unknown demo dataset" in r.stderr
