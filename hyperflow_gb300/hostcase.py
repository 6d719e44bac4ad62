"""Case and result files of the C host program `hf_host_run` (host/hf_host_run.c), which
drives the stepper through the C ABI only (the BlockAMR::run loop of
HyperFlow_V3/src/BlockAMR.cpp:400-423 for a uniform single-patch level)."""
import os
import struct
import subprocess

import numpy as np

from . import _lib as L
from .build import HOST_BIN

_BC = {"reflecting": L.HF_BC_REFLECTING, "transmissive": L.HF_BC_TRANSMISSIVE, "inflow": L.HF_BC_INFLOW,
       "wedge": L.HF_BC_WEDGE}


def write_case(path, U, nx, ny, dx, dy, nsteps, mechanism="H2_Li", xlo=0.0, ylo=0.0, periodic=(0, 0),
               boundary_lo=("reflecting", "reflecting"), boundary_hi=("transmissive", "reflecting"), inlet=None,
               wedge_start=0.0, cfl=0.5, rtol=1e-8, atol=1e-15, flux=L.HF_FLUX_PLAIN,
               chem=L.HF_CHEM_PERSISTENT, chemistry=True):
    """U: (NV, ny, nx) float64 initial state; the level keys are those of make_level."""
    U = np.ascontiguousarray(U, dtype=np.float64)
    if U.shape[1:] != (ny, nx):
        raise ValueError("state shape %s does not match the level %d x %d" % (U.shape, nx, ny))
    inl = np.zeros(13)
    if inlet is not None:
        inl[:len(inlet)] = inlet
    ints = [nx, ny, int(periodic[0]), int(periodic[1]), _BC[boundary_lo[0]], _BC[boundary_lo[1]],
            _BC[boundary_hi[0]], _BC[boundary_hi[1]], int(nsteps), int(flux), int(chem), int(bool(chemistry))]
    dbl = [dx, dy, xlo, ylo, wedge_start, cfl, rtol, atol] + list(inl)
    with open(path, "wb") as f:
        f.write(b"HFCASE1\0")
        f.write(struct.pack("=12i", *ints))
        f.write(struct.pack("=21d", *dbl))
        f.write(mechanism.encode().ljust(32, b"\0"))
        f.write(U.tobytes())


def read_result(path, nv, ny, nx, nsteps):
    """(steps taken, final time, step sizes (nsteps,), final state (NV, ny, nx))."""
    with open(path, "rb") as f:
        taken, = struct.unpack("=i", f.read(4))
        t, = struct.unpack("=d", f.read(8))
        dts = np.frombuffer(f.read(8 * nsteps), dtype=np.float64).copy()
        U = np.frombuffer(f.read(8 * nv * ny * nx), dtype=np.float64).reshape(nv, ny, nx).copy()
    return taken, t, dts, U


def run(case_path, result_path):
    """Run hf_host_run; returns the completed process (returncode 0 = success)."""
    if not os.path.exists(HOST_BIN):
        raise OSError("hf_host_run is not built: run hyperflow_gb300.build.build() first")
    return subprocess.run([HOST_BIN, case_path, result_path], capture_output=True, text=True)
