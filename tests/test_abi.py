"""The C ABI: the library builds, loads without a GPU and exports every symbol
include/gpgp.h declares; struct layouts match the header. CPU only."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gpgp.h")
LIB = os.path.join(ROOT, "gplite_gb300", "libgpgp.so")


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(gpgp_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB):
        from gplite_gb300 import build
        build.build()
    return C.CDLL(LIB)


def test_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s


def test_binding_covers_header():
    from gplite_gb300 import _lib
    assert set(declared_symbols()) <= set(_lib.SIGNATURES)


def test_struct_sizes_match_c(lib):
    """Compile a tiny C program against the header and compare sizeof/offsetof with ctypes."""
    import subprocess
    import tempfile
    from gplite_gb300 import _lib as L
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "gpgp.h"
int main(void){
 printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(gpgp_cf_term),
  sizeof(gpgp_kernel), sizeof(gpgp_lik), sizeof(gpgp_method), sizeof(gpgp_approx), sizeof(gpgp_fit_opts),
  sizeof(gpgp_fit_result), offsetof(gpgp_cf_term, lscale), sizeof(gpgp_batch_problem),
  sizeof(gpgp_server_opts), sizeof(gpgp_request), offsetof(gpgp_request, model), sizeof(gpgp_request_result),
  sizeof(gpgp_server_stats), offsetof(gpgp_server_stats, p50_ms));
 return 0;}
'''
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "s.c")
        open(p, "w").write(src)
        exe = os.path.join(d, "s")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), p, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    got = [C.sizeof(L.CfTerm), C.sizeof(L.Kernel), C.sizeof(L.Lik), C.sizeof(L.Method),
           C.sizeof(L.Approx), C.sizeof(L.FitOpts), C.sizeof(L.FitResult), L.CfTerm.lscale.offset,
           C.sizeof(L.BatchProblem), C.sizeof(L.ServerOpts), C.sizeof(L.Request), L.Request.model.offset,
           C.sizeof(L.RequestResult), C.sizeof(L.ServerStats), L.ServerStats.p50_ms.offset]
    assert [int(v) for v in out] == got


def test_status_strings(lib):
    lib.gpgp_status_string.restype = C.c_char_p
    assert lib.gpgp_status_string(0) == b"ok"
    assert lib.gpgp_status_string(1).startswith(b"matrix not positive")


def test_create_without_gpu_fails_cleanly(lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except Exception:
        pass
    h = C.c_void_p()
    st = lib.gpgp_create(C.byref(h), 0)
    assert st != 0 and not h.value
