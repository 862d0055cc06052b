"""Builds voxhenry_gpu_mex.c against the stub mex.h (either complex layout) and calls it from Python:
the MATLAB side of the MEX gateway, without MATLAB (test infrastructure)."""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
PKG = os.path.join(ROOT, "voxhenry_gb300")


def build(outdir: str, interleaved: bool) -> str:
    so = os.path.join(outdir, f"gateway_{'interleaved' if interleaved else 'split'}.so")
    cmd = ["gcc", "-std=c99", "-O1", "-fPIC", "-shared", "-Wall", "-Wextra", "-Wno-unused-parameter", "-Werror",
           "-I", HERE, "-I", os.path.join(ROOT, "include"), os.path.join(PKG, "mex", "voxhenry_gpu_mex.c"),
           os.path.join(HERE, "mex_stub.c"), "-L", PKG, "-lvhgpu", f"-Wl,-rpath,{PKG}", "-o", so]
    if interleaved:
        cmd.insert(1, "-DMX_HAS_INTERLEAVED_COMPLEX")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    return so


class MexError(RuntimeError):
    def __init__(self, text):
        ident, _, msg = text.partition("|")
        super().__init__(f"{ident}: {msg}")
        self.identifier = ident


class Gateway:
    """voxhenry_gpu_mex as MATLAB would call it: numpy arrays in, numpy arrays out."""

    def __init__(self, so_path):
        self.lib = C.CDLL(so_path)
        L = self.lib
        L.stub_double.restype = C.c_void_p
        L.stub_double.argtypes = [C.c_int, C.POINTER(C.c_longlong), C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.stub_sparse.restype = C.c_void_p
        L.stub_sparse.argtypes = [C.c_longlong, C.c_longlong, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong),
                                  C.POINTER(C.c_double)]
        L.stub_char.restype = C.c_void_p
        L.stub_char.argtypes = [C.c_char_p]
        L.stub_numel.restype = C.c_size_t
        L.stub_numel.argtypes = [C.c_void_p]
        L.stub_read.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.stub_free.argtypes = [C.c_void_p]
        L.stub_call.argtypes = [C.c_int, C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_void_p)]
        L.stub_error.restype = C.c_char_p
        self.interleaved = bool(L.stub_interleaved())

    def _arg(self, v):
        import scipy.sparse as sp

        L = self.lib
        if isinstance(v, str):
            return L.stub_char(v.encode())
        if sp.issparse(v):
            A = sp.csc_matrix(v)
            A.sort_indices()
            jc = np.ascontiguousarray(A.indptr, dtype=np.longlong)
            ir = np.ascontiguousarray(A.indices, dtype=np.longlong)
            pr = np.ascontiguousarray(A.data, dtype=np.float64)
            return L.stub_sparse(A.shape[0], A.shape[1], jc.ctypes.data_as(C.POINTER(C.c_longlong)),
                                 ir.ctypes.data_as(C.POINTER(C.c_longlong)), pr.ctypes.data_as(C.POINTER(C.c_double)))
        a = np.asarray(v)
        if a.ndim == 0:
            a = a.reshape(1, 1)
        elif a.ndim == 1:
            a = a.reshape(-1, 1)
        dims = np.asarray(a.shape, dtype=np.longlong)
        re = np.ascontiguousarray(a.real.ravel(order="F"), dtype=np.float64)
        im = np.ascontiguousarray(a.imag.ravel(order="F"), dtype=np.float64) if np.iscomplexobj(a) else None
        return L.stub_double(a.ndim, dims.ctypes.data_as(C.POINTER(C.c_longlong)),
                             re.ctypes.data_as(C.POINTER(C.c_double)),
                             im.ctypes.data_as(C.POINTER(C.c_double)) if im is not None else None)

    def _out(self, p):
        n = self.lib.stub_numel(p)
        re = np.zeros(n)
        im = np.zeros(n)
        self.lib.stub_read(p, re.ctypes.data_as(C.POINTER(C.c_double)), im.ctypes.data_as(C.POINTER(C.c_double)))
        self.lib.stub_free(p)
        return re + 1j * im if np.any(im) else re

    def __call__(self, *args, nargout=1):
        prhs = (C.c_void_p * len(args))(*[self._arg(a) for a in args])
        plhs = (C.c_void_p * max(1, nargout))()
        try:
            if self.lib.stub_call(nargout, plhs, len(args), prhs):
                raise MexError(self.lib.stub_error().decode())
        finally:
            for p in prhs:
                self.lib.stub_free(p)
        outs = [self._out(p) for p in plhs[:nargout] if p]
        return outs[0] if nargout == 1 else outs

    def exit(self):
        self.lib.stub_exit()
