"""The C host program hf_host_run (host/hf_host_run.c): a plain-C99 caller of the C ABI.
CPU checks: it builds with the library, reports usage and I/O errors with exit status 2
before touching a GPU, and the case file has the layout the program reads."""
import os
import struct
import subprocess

import numpy as np


def test_host_program_usage_and_io_errors(tmp_path):
    from hyperflow_gb300 import build
    build.build()
    r = subprocess.run([build.HOST_BIN], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
    r = subprocess.run([build.HOST_BIN, str(tmp_path / "missing"), str(tmp_path / "out")], capture_output=True,
                       text=True)
    assert r.returncode == 2 and "cannot open" in r.stderr
    bad = tmp_path / "bad"
    bad.write_bytes(b"NOTACASE" + bytes(200))
    r = subprocess.run([build.HOST_BIN, str(bad), str(tmp_path / "out")], capture_output=True, text=True)
    assert r.returncode == 2 and "header" in r.stderr


def test_case_file_layout(tmp_path):
    from hyperflow_gb300 import hostcase
    from hyperflow_gb300 import workloads as W
    U, lvd = W.det2d(seed=2, diluent="N2", nx=16, ny=4, hot_columns=4)
    path = str(tmp_path / "case")
    hostcase.write_case(path, U, nsteps=3, mechanism="H2_Li", **lvd)
    raw = open(path, "rb").read()
    assert raw[:8] == b"HFCASE1\0"
    ints = struct.unpack("=12i", raw[8:56])
    assert ints[:2] == (16, 4) and ints[2:4] == (0, 1) and ints[8] == 3
    dbl = struct.unpack("=21d", raw[56:224])
    assert dbl[0] == lvd["dx"] and dbl[5] == 0.5 and np.array_equal(dbl[8:20], lvd["inlet"])
    assert raw[224:256].rstrip(b"\0") == b"H2_Li"
    assert np.array_equal(np.frombuffer(raw[256:], dtype=np.float64).reshape(U.shape), U)
