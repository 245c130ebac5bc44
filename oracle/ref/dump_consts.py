#!/usr/bin/env python3
"""Writes oracle/_ref/ref_consts_<N>.bin: the device constant tables of the
reference library for the moduli set of N moduli, as its own rns_const_init()
and mp_const_init() (src/rns.cuh:324-442, src/arith/arith_utils.cuh:44-90)
compute them on the host with GMP/MPFR and upload them with
cudaMemcpyToSymbol.  Read from the CPU build oracle/_ref/libmpres_ref_<N>.so
after its init, where those uploads land in host copies of the same `cuda::`
symbols.  oracle/ref_gpu.py fills the same symbols of the reference's cubin
from this file on the GPU.  TEST AND BENCHMARK INFRASTRUCTURE ONLY.

Format: b"MPRC", u32 count, then per symbol u16 name length, the mangled
name, u32 byte size, the bytes.

    python oracle/ref/dump_consts.py 8 16 32
"""
import ctypes
import pathlib
import struct
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
REF = HERE.parent / "_ref"
SKIP = {"_ZN4cuda5sdataE"}  # the CPU build's stand-in for dynamic shared memory


def dump(n):
    so = REF / ("libmpres_ref_%d.so" % n)
    lib = ctypes.CDLL(str(so))
    lib.ref_init()
    out = subprocess.run(["nm", "-DS", str(so)], capture_output=True, text=True, check=True).stdout
    syms = []
    for line in out.splitlines():
        parts = line.split()
        if len(parts) == 4 and parts[2] in ("B", "D") and parts[3].startswith("_ZN4cuda") and parts[3] not in SKIP:
            syms.append((parts[3], int(parts[1], 16)))
    blob = bytearray(b"MPRC" + struct.pack("<I", len(syms)))
    for name, size in sorted(syms):
        data = bytes((ctypes.c_char * size).in_dll(lib, name))
        blob += struct.pack("<H", len(name)) + name.encode() + struct.pack("<I", size) + data
    (REF / ("ref_consts_%d.bin" % n)).write_bytes(bytes(blob))
    return len(syms)


if __name__ == "__main__":
    for a in sys.argv[1:] or ["8", "16", "32"]:
        print("ref_consts_%s.bin: %d symbols" % (a, dump(int(a))))
