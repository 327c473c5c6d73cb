"""Comparators for bench.py: Photon's Kokkos BVH ray back-end restated for
the GPU, and an L2 read-bandwidth probe.

kokkos_port.cu restates the reference's KokkosBackend (binary median-split
BVH, one thread per ray with a 64-entry stack, 88-byte HitResult records;
src/photon/pt/backend/kokkos_backend.cpp:21-86) as it runs under Kokkos-CUDA.
It exists only to time the reference's Level-A algorithm beside this
library's BVH8 back-end on the same GPU and rays; the library never uses it.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRCS = [os.path.join(HERE, "kokkos_port.cu"), os.path.join(HERE, "l2_probe.cu")]
LIB = os.path.join(HERE, "_build", "libkokkos_port.so")
_lib = None


def build(force: bool = False) -> str:
    """nvcc, sm_103a; device code with nvcc's default contraction (as the
    reference's Kokkos-CUDA build), host code without (-ffp-contract=off, so
    the host traversal rounds like the CPU oracle)."""
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(s) for s in SRCS):
        return LIB
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-lineinfo",
           "-Xcompiler", "-fPIC,-ffp-contract=off", "-shared", "-o", LIB] + SRCS
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"kokkos_port build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(LIB)
        lib.kbp_error.restype = C.c_char_p
        lib.kbp_create.argtypes = [C.POINTER(C.c_void_p), C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64,
                                   C.c_void_p, C.c_void_p, C.c_int]
        lib.kbp_destroy.argtypes = [C.c_void_p]
        lib.kbp_info.argtypes = [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        lib.kbp_trace.argtypes = [C.c_void_p] + [C.c_void_p] * 4 + [C.c_uint32, C.c_int, C.c_void_p, C.c_void_p]
        lib.kbp_trace_host.argtypes = [C.c_void_p] + [C.c_void_p] * 4 + [C.c_uint32, C.c_int, C.c_void_p]
        lib.kbp_loop_overhead_us.restype = C.c_double
        lib.kbp_loop_overhead_us.argtypes = [C.c_int]
        lib.l2_read_gbs.restype = C.c_double
        lib.l2_read_gbs.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_void_p]
        _lib = lib
    return _lib


class KokkosPortAccel:
    """The reference's BVH over an indexed mesh (host build; `device` copies
    it to the current GPU)."""

    def __init__(self, positions, indices, normals=None, material_ids=None, device=True):
        self.lib = load()
        self._pos = np.ascontiguousarray(positions, np.float32).reshape(-1)
        self._idx = np.ascontiguousarray(indices, np.uint32).reshape(-1)
        self._nrm = None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(-1)
        self._mid = None if material_ids is None else np.ascontiguousarray(material_ids, np.uint32).reshape(-1)
        h = C.c_void_p()
        rc = self.lib.kbp_create(C.byref(h), self._pos.ctypes.data, self._pos.size // 3, self._idx.ctypes.data,
                                 self._idx.size // 3, None if self._nrm is None else self._nrm.ctypes.data,
                                 None if self._mid is None else self._mid.ctypes.data, int(device))
        if rc != 0:
            raise RuntimeError(self.lib.kbp_error().decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.kbp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        n, d = C.c_uint64(), C.c_uint64()
        self.lib.kbp_info(self.h, C.byref(n), C.byref(d))
        return {"nodes": n.value, "depth": d.value}

    def trace(self, o, d, tmin, tmax, out, any_hit=False, stream=None):
        """Device tensors: o, d (n, 3) float32, tmin/tmax (n,), out (n, 88)
        uint8 (closest) or (n,) int32 (any hit).  Asynchronous on `stream`
        (a cudaStream_t handle, None: the legacy default stream)."""
        rc = self.lib.kbp_trace(self.h, o.data_ptr(), d.data_ptr(), tmin.data_ptr(), tmax.data_ptr(),
                                int(tmin.numel()), int(any_hit), out.data_ptr(), stream)
        if rc != 0:
            raise RuntimeError(self.lib.kbp_error().decode())
        return out

    def trace_host(self, o, d, tmin, tmax, any_hit=False):
        """The same traversal on the CPU over numpy arrays; HitResult records
        (photon_gb300._abi.hit_dtype) or u32 occlusion flags."""
        from photon_gb300 import _abi
        o = np.ascontiguousarray(o, np.float32)
        d = np.ascontiguousarray(d, np.float32)
        t0 = np.ascontiguousarray(tmin, np.float32)
        t1 = np.ascontiguousarray(tmax, np.float32)
        n = len(t0)
        out = np.zeros(n, np.uint32) if any_hit else np.zeros(n, _abi.hit_dtype())
        rc = self.lib.kbp_trace_host(self.h, o.ctypes.data, d.ctypes.data, t0.ctypes.data, t1.ctypes.data, n,
                                     int(any_hit), out.ctypes.data)
        if rc != 0:
            raise RuntimeError(self.lib.kbp_error().decode())
        return out


def l2_read_gbs(mib: int = 32, reps: int = 64) -> float:
    """Read bandwidth (GB/s) of a `mib` MiB device buffer swept `reps` times in
    one launch (l2_probe.cu): with the buffer far below the 129 MB L2 this is
    the L2 ceiling of an L2-resident traversal."""
    import torch
    lib = load()
    buf = torch.ones(mib * 2 ** 20 // 4, dtype=torch.float32, device="cuda")
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    blocks = sms * 8
    sink = torch.empty(blocks * 256, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    best = max(lib.l2_read_gbs(buf.data_ptr(), buf.numel() * 4, reps, blocks, sink.data_ptr()) for _ in range(3))
    if best <= 0:
        raise RuntimeError("l2 probe failed")
    return best


def loop_overhead_s(reps: int = 300) -> float:
    """Fixed cost in seconds of one bounce iteration of the reference's render
    loop on this GPU and host (kokkos_port.cu kbp_loop_overhead_us: five empty
    launches, two synchronisations, one 4-byte read-back from C++)."""
    us = load().kbp_loop_overhead_us(int(reps))
    if us <= 0:
        raise RuntimeError("loop overhead probe failed")
    return us * 1e-6
