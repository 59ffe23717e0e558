"""The tensor-network mode's batched real GEMM (tedq_tn_gemm, the kernel each
large pairwise contraction runs) against a float64 torch product, through the
C ABI: the tcgen05 tensor-core kernel with the 3xTF32 split (FP32 accuracy)
and with one TF32 product, the FP32 and FP64 FMA kernels.  Shapes cover the
6x6-lattice contractions (both orientations: the larger side fills the
128-row tiles), partial tiles in every dimension, K not a multiple of the
stage's K-block (8, 16 or 32 elements with 32-, 64- and 128-byte swizzles),
shared (unbatched) operands and the error word.

Tolerance: |C - C64| <= tol * sqrt(kr) * max|A| * max|B| with tol = 2e-6
(3xTF32, FP32), 2e-3 (TF32), 1e-13 (FP64)."""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

qai = pytest.importorskip("tedq_gb300")
from tedq_gb300 import _lib  # noqa: E402

DEV = "cuda:0"
MODES = {"fp32": 0, "tc32": 1, "tf32": 2, "auto": 3}

# (mr, nr, kr) of the 6x6x8 lattice's large contractions, then edge cases
SHAPES = [(64, 128, 8), (32, 256, 8), (64, 128, 16), (128, 256, 64), (64, 128, 256), (64, 512, 16),
          (128, 1024, 32), (128, 1024, 128), (256, 512, 256), (32, 256, 512),
          (200, 40, 12), (40, 200, 44), (130, 17, 36), (512, 8, 100), (96, 96, 4 * 33), (64, 96, 4),
          (128, 64, 12), (300, 24, 16)]


def _run(mode, prec, mr, nr, kr, nbatch, shared_a=False, shared_b=False, seed=0):
    g = torch.Generator().manual_seed(seed)
    dt = torch.float64 if prec == "c128" else torch.float32
    A = torch.rand(1 if shared_a else nbatch, mr, kr, generator=g, dtype=torch.float64) * 2 - 1
    B = torch.rand(1 if shared_b else nbatch, nr, kr, generator=g, dtype=torch.float64) * 2 - 1
    want = torch.einsum("bik,bjk->bji", A.expand(nbatch, mr, kr), B.expand(nbatch, nr, kr))  # C[b][j][i]
    Ad, Bd = A.to(DEV, dt).contiguous(), B.to(DEV, dt).contiguous()
    C = torch.full((nbatch, nr, mr), float("nan"), dtype=dt, device=DEV)
    err = torch.zeros(1, dtype=torch.int32, device=DEV)
    st = _lib.lib().tedq_tn_gemm(
        _lib.PREC_C128 if prec == "c128" else _lib.PREC_C64, MODES[mode], ctypes.c_void_p(Ad.data_ptr()),
        ctypes.c_void_p(Bd.data_ptr()), ctypes.c_void_p(C.data_ptr()), mr, nr, kr, 0 if shared_a else mr * kr,
        0 if shared_b else nr * kr, nr * mr, nbatch, ctypes.c_void_p(err.data_ptr()),
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(st, "tedq_tn_gemm")
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    scale = float(np.sqrt(kr))
    return C.double().cpu(), want, scale


TOL = {"tc32": 2e-6, "fp32": 2e-6, "tf32": 2e-3}


@pytest.mark.parametrize("mode", ["tc32", "tf32", "fp32"])
@pytest.mark.parametrize("shape", SHAPES, ids=[f"{m}x{n}x{k}" for m, n, k in SHAPES])
def test_gemm_matches_float64(shape, mode):
    mr, nr, kr = shape
    nb = 3
    got, want, scale = _run(mode, "c64", mr, nr, kr, nb, seed=mr + nr + kr)
    assert torch.isfinite(got).all()
    assert (got - want).abs().max().item() <= TOL[mode] * scale


@pytest.mark.parametrize("shared", [(True, False), (False, True)], ids=["shared_a", "shared_b"])
def test_gemm_shared_operand(shared):
    got, want, scale = _run("tc32", "c64", 128, 64, 64, 4, shared_a=shared[0], shared_b=shared[1], seed=9)
    assert (got - want).abs().max().item() <= TOL["tc32"] * scale


def test_gemm_fp64():
    got, want, scale = _run("fp32", "c128", 96, 130, 72, 2, seed=4)
    assert (got - want).abs().max().item() <= 1e-13 * scale


def test_gemm_large_batch_and_auto():
    """The benchmark's largest contraction shape at batch 256, AUTO mode."""
    got, want, scale = _run("auto", "c64", 256, 512, 256, 256, seed=5)
    assert (got - want).abs().max().item() <= TOL["tc32"] * scale


def test_gemm_rejects_unsupported_tensor_core_shape():
    A = torch.zeros(8, 6, device=DEV)
    C = torch.zeros(8, 8, device=DEV)
    err = torch.zeros(1, dtype=torch.int32, device=DEV)
    # kr = 6: rows of 24 bytes cannot be TMA-strided (16-byte multiples)
    st = _lib.lib().tedq_tn_gemm(_lib.PREC_C64, MODES["tc32"], ctypes.c_void_p(A.data_ptr()),
                                 ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(C.data_ptr()), 8, 8, 6, 0, 0, 0, 1,
                                 ctypes.c_void_p(err.data_ptr()), None)
    assert st == _lib.ERR_UNSUPPORTED


@pytest.mark.parametrize("prec", ["c64", "c128"])
def test_gemm_tiny_output_long_sum(prec):
    """The closing contraction shape (1 x 2 outputs over 8192 terms) runs on
    the block-reduction kernel."""
    got, want, scale = _run("auto" if prec == "c64" else "fp32", prec, 1, 2, 8192, 5, seed=8)
    assert (got - want).abs().max().item() <= (2e-6 if prec == "c64" else 1e-13) * scale
