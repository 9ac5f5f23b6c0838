"""Device algorithms compiled for the host and checked block by block against
the oracle: CPU parity checks of the GPU code itself.

* The per-thread RS256 decoder of the table path (rs256_device.cuh: LFSR
  remainder, syndromes, Berlekamp-Massey, Chien search, Forney) over ecc
  1..254, shortened blocks and error counts past the capacity.
* The RSi16 register transforms (rsi16_device.cuh: the sub-warp syndromes and
  encodes for ecc 2..16, the two-block register ones for ecc 32 and 64) and
  the RSi16 repair paths (lane-per-block Berlekamp-Massey batches, the
  per-block bounded-distance path, the step-for-step mirror, known positions)
  on the oracle's own code tables, with the warp emulated by 32 host threads
  in lock step.
* The lazily reduced arithmetic of the one-block-per-thread RSi16 kernels
  (rsi16_bt.cuh, ecc 32 and 64): parity, syndromes and the lane
  Berlekamp-Massey.
* The nibble-table RS256 encoder (rs256_nib.cuh): its tables and lane code."""

import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("g++") is None or shutil.which("gcc") is None, reason="needs gcc/g++")
def test_rs256_device_decoder_on_host(tmp_path):
    obj = tmp_path / "ffrs_oracle.o"
    exe = tmp_path / "rs256_solve_check"
    subprocess.run(["gcc", "-O2", "-c", os.path.join(REPO, "oracle", "ffrs_oracle.c"), "-o", str(obj)], check=True)
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(REPO, "tests", "host", "stub"),
                    "-I", os.path.join(REPO, "libffrs_gb300", "csrc"), "-I", os.path.join(REPO, "oracle"),
                    os.path.join(REPO, "tests", "host", "rs256_solve_check.cpp"), str(obj), "-o", str(exe)],
                   check=True)
    r = subprocess.run([str(exe), "11", "3000"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("bad 0"), r.stdout[-2000:]


@pytest.mark.skipif(shutil.which("g++") is None or shutil.which("gcc") is None, reason="needs gcc/g++")
def test_rsi16_transforms_on_host(tmp_path):
    obj = tmp_path / "ffrs_oracle.o"
    exe = tmp_path / "rsi16_transform_check"
    subprocess.run(["gcc", "-O2", "-c", os.path.join(REPO, "oracle", "ffrs_oracle.c"), "-o", str(obj)], check=True)
    subprocess.run(["g++", "-O2", "-std=c++20", "-pthread", "-I", os.path.join(REPO, "tests", "host", "stub"),
                    "-I", os.path.join(REPO, "libffrs_gb300", "csrc"), "-I", os.path.join(REPO, "oracle"),
                    os.path.join(REPO, "tests", "host", "rsi16_transform_check.cpp"), str(obj), "-o", str(exe)],
                   check=True)
    r = subprocess.run([str(exe), "17", "64"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("bad 0"), r.stdout[-2000:]


@pytest.mark.skipif(shutil.which("g++") is None or shutil.which("gcc") is None, reason="needs gcc/g++")
def test_rsi16_repairs_on_host(tmp_path):
    obj = tmp_path / "ffrs_oracle.o"
    exe = tmp_path / "rsi16_repair_check"
    subprocess.run(["gcc", "-O2", "-c", os.path.join(REPO, "oracle", "ffrs_oracle.c"), "-o", str(obj)], check=True)
    subprocess.run(["g++", "-O2", "-std=c++20", "-pthread", "-I", os.path.join(REPO, "tests", "host", "stub"),
                    "-I", os.path.join(REPO, "libffrs_gb300", "csrc"), "-I", os.path.join(REPO, "oracle"),
                    os.path.join(REPO, "tests", "host", "rsi16_repair_check.cpp"), str(obj), "-o", str(exe)],
                   check=True)
    r = subprocess.run([str(exe), "19", "3"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("bad 0"), r.stdout[-2000:]


@pytest.mark.skipif(shutil.which("g++") is None or shutil.which("gcc") is None, reason="needs gcc/g++")
def test_rs256_syndrome_networks_on_host(tmp_path):
    """The generated bitsliced syndrome networks (rs256_synd_gen.cuh) against
    the oracle's syndromes, full and shortened blocks."""
    obj = tmp_path / "ffrs_oracle.o"
    exe = tmp_path / "rs256_synd_check"
    subprocess.run(["gcc", "-O2", "-c", os.path.join(REPO, "oracle", "ffrs_oracle.c"), "-o", str(obj)], check=True)
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(REPO, "tests", "host", "stub"),
                    "-I", os.path.join(REPO, "libffrs_gb300", "csrc"), "-I", os.path.join(REPO, "oracle"),
                    os.path.join(REPO, "tests", "host", "rs256_synd_check.cpp"), str(obj), "-o", str(exe)],
                   check=True)
    r = subprocess.run([str(exe), "5", "300"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("bad 0"), r.stdout[-2000:]


def test_generated_syndrome_header_is_current():
    """rs256_synd_gen.cuh is exactly what gen_rs256_synd.py emits."""
    import importlib.util

    path = os.path.join(REPO, "libffrs_gb300", "csrc", "gen_rs256_synd.py")
    spec = importlib.util.spec_from_file_location("gen_rs256_synd", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    with open(mod.OUT) as f:
        assert f.read() == mod.generate()


@pytest.mark.skipif(shutil.which("g++") is None or shutil.which("gcc") is None, reason="needs gcc/g++")
def test_rsi16_block_per_thread_arithmetic_on_host(tmp_path):
    """The lazily reduced transforms and Berlekamp-Massey of the one-block-per-
    thread RSi16 kernels (rsi16_bt.cuh): parity, syndromes and the lane
    Berlekamp-Massey against the oracle, ecc 32 and 64, up to 65536 words."""
    obj = tmp_path / "ffrs_oracle.o"
    exe = tmp_path / "rsi16_bt_check"
    subprocess.run(["gcc", "-O2", "-c", os.path.join(REPO, "oracle", "ffrs_oracle.c"), "-o", str(obj)], check=True)
    subprocess.run(["g++", "-O2", "-std=c++20", "-pthread", "-I", os.path.join(REPO, "tests", "host", "stub"),
                    "-I", os.path.join(REPO, "libffrs_gb300", "csrc"), "-I", os.path.join(REPO, "oracle"),
                    os.path.join(REPO, "tests", "host", "rsi16_bt_check.cpp"), str(obj), "-o", str(exe)],
                   check=True)
    r = subprocess.run([str(exe), "23", "96"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("bad 0"), r.stdout[-2000:]


@pytest.mark.skipif(shutil.which("g++") is None or shutil.which("gcc") is None, reason="needs gcc/g++")
def test_rs256_nibble_encoder_on_host(tmp_path):
    """The nibble-table RS256 encoder's tables and lane code (rs256_nib.cuh)
    against the oracle's encode: message lengths 1..223, buffers 0/4/8/12
    bytes past a 16-byte boundary, poison around the staged table and the
    buffer."""
    obj = tmp_path / "ffrs_oracle.o"
    exe = tmp_path / "rs256_nib_check"
    subprocess.run(["gcc", "-O2", "-c", os.path.join(REPO, "oracle", "ffrs_oracle.c"), "-o", str(obj)], check=True)
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(REPO, "tests", "host", "stub"),
                    "-I", os.path.join(REPO, "libffrs_gb300", "csrc"), "-I", os.path.join(REPO, "oracle"),
                    os.path.join(REPO, "tests", "host", "rs256_nib_check.cpp"), str(obj), "-o", str(exe)],
                   check=True)
    r = subprocess.run([str(exe), "29", "96"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("bad 0"), r.stdout[-2000:]
