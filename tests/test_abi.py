"""CPU tests of the C-ABI boundary: the library loads and exports every
symbol include/flock_gb300.h declares, host-side logic agrees with the oracle,
and host-side rejections return the documented codes without touching a GPU."""
from __future__ import annotations

import ctypes as C
import subprocess

import numpy as np
import pytest


def test_library_exports_every_declared_symbol(native):
    syms = native.header_symbols()
    assert len(syms) >= 30
    L = C.CDLL(native.LIB_PATH)
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing


def test_no_oracle_in_the_product(native):
    # the product library must not link or embed the oracle
    out = subprocess.run(["nm", "-D", native.LIB_PATH], capture_output=True, text=True).stdout
    assert "orc_" not in out


@pytest.mark.parametrize("n,seed", [(0, 1), (1, 1), (2000, 1), (100_000, 1), (4321, 7), (1000, 3)])
def test_generator_matches_the_oracle_bit_for_bit(native, oracle, n, seed):
    assert native.generate(n, seed).tobytes() == oracle.scatter(n, seed).tobytes()


def test_constants_match_the_oracle_word_for_word(native, oracle):
    a = np.array(list(native.params().values()), dtype=np.float32)
    assert list(native.params()) == list(oracle.params())
    assert a.tobytes() == oracle.params_raw().tobytes()


def test_buckets_for_agrees(native, oracle):
    for n in [0, 1, 999, 32768, 32769, 65536, 100_000, 1_000_000, 2_097_152, 16_777_216, 40_000_000]:
        assert native.buckets_for(n) == oracle.buckets_for(n)


def test_bytes_for_grows_with_n(native):
    assert native.bytes_for(1000) < native.bytes_for(100_000) < native.bytes_for(1_000_000)
    assert native.bytes_for(1_000_000) < 300 * 1_000_000
    assert native.kernels_per_step() == 6


def test_open_file_rejections_happen_on_the_host(native, tmp_path):
    m = native
    with pytest.raises(m.FlockError) as e:
        m.Flock.open(str(tmp_path / "missing.flk"))
    assert e.value.code == -2 and "cannot open" in str(e.value)
    # through the C ABI directly (no Python format helper in between)
    h = C.c_void_p()
    rc = m.lib().flk_open_file(-1, str(tmp_path / "missing.flk").encode(), C.byref(h))
    assert rc == -2 and b"cannot open" in m.lib().flk_last_error()
    bad = tmp_path / "bad.flk"
    bad.write_bytes(b"FLK2" + bytes(12))
    assert m.lib().flk_open_file(-1, str(bad).encode(), C.byref(h)) == -7
    words = tmp_path / "words.flk"
    words.write_bytes(b"FLK1" + np.array([1, 14], "<u4").tobytes() + bytes(4) + bytes(56))
    assert m.lib().flk_open_file(-1, str(words).encode(), C.byref(h)) == -7
    trunc = tmp_path / "trunc.flk"
    trunc.write_bytes(b"FLK1" + np.array([3, 15], "<u4").tobytes() + bytes(4) + bytes(60))
    assert m.lib().flk_open_file(-1, str(trunc).encode(), C.byref(h)) == -2
    assert b"truncated" in m.lib().flk_last_error()
    assert m.lib().flk_open_host(-1, 5, 0.0, None, C.byref(h)) == -1
    assert m.lib().flk_step(None, 1) == -1
    assert m.lib().flk_read_host(None, None, None) == -1


def test_cli_usage_errors(native, tmp_path):
    r = subprocess.run([native.CLI_PATH], capture_output=True, text=True)
    assert r.returncode == 2 and "missing --in" in r.stderr
    r = subprocess.run([native.CLI_PATH, "--bogus"], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
    r = subprocess.run([native.CLI_PATH, "--in"], capture_output=True, text=True)
    assert r.returncode == 2
    r = subprocess.run([native.CLI_PATH, "--in", str(tmp_path / "none.flk")], capture_output=True, text=True)
    assert r.returncode == 1


def test_python_flk_helpers_match_the_oracle_writer(native, oracle, tmp_path):
    w = oracle.scatter(77, 9)
    p1, p2 = str(tmp_path / "a.flk"), str(tmp_path / "b.flk")
    native.write_flk(p1, 0.125, w)
    subprocess.run([oracle.CLI, "gen", "--birds", "77", "--seed", "9", "--out", p2], check=True)
    t, back = native.read_flk(p2)
    assert t == 0.0 and back.tobytes() == w.tobytes()
    raw1 = open(p1, "rb").read()
    raw2 = open(p2, "rb").read()
    assert raw1[:12] == raw2[:12] and raw1[16:] == raw2[16:]
    with pytest.raises(ValueError):
        bad = tmp_path / "x.flk"
        bad.write_bytes(b"nope")
        native.read_flk(str(bad))


def test_file_info_reads_the_header(native, tmp_path):
    w = native.generate(123, 5)
    path = str(tmp_path / "x.flk")
    native.write_flk(path, 0.375, w)
    assert native.file_info(path) == (123, 0.375)
    with pytest.raises(native.FlockError) as e:
        native.file_info(str(tmp_path / "missing.flk"))
    assert e.value.code == -2
    bad = tmp_path / "bad.flk"
    bad.write_bytes(b"FLK2" + bytes(12))
    with pytest.raises(native.FlockError) as e:
        native.file_info(str(bad))
    assert e.value.code == -7


def test_header_is_plain_c(native, tmp_path):
    """include/flock_gb300.h is the FFI boundary: it compiles as strict C99 (what
    bindgen, cgo or a C caller sees) and as C++."""
    import os
    import shutil

    hdr_dir = os.path.dirname(native.HEADER)
    src = tmp_path / "use.c"
    src.write_text('#include "flock_gb300.h"\nint main(void) { return flk_buckets_for(10) == 0; }\n')
    for cc, extra in (("gcc", ["-std=c99", "-pedantic", "-Werror"]), ("g++", ["-x", "c++", "-std=c++11", "-Werror"])):
        if shutil.which(cc) is None:
            pytest.skip(f"{cc} not available")
        r = subprocess.run([cc, *extra, "-Wall", "-Wextra", "-I" + hdr_dir, "-c", str(src), "-o",
                            str(tmp_path / "use.o")], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_device_error_words_map_to_their_messages(native):
    # what FLK_ERR_DEVICE reports for each device error word (no GPU involved)
    assert "scan look-back wait gave up" in native.device_error_text(1)
    assert "outside its array" in native.device_error_text(2)
    assert native.device_error_text(0) == "no device error"
    assert native.device_error_text(77) == "unknown device error word"
