"""The split-FP16 tcgen05 GEMM engine (descriptors, tensor memory, bulk
copies, commit/wait) against a float64 product: with hi+lo operands and FP32
accumulation the result carries about 22 significant bits, so every element
must be within a few 1e-6 of the row's scale."""
import numpy as np
import pytest

import xcorr_gb300 as xg

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.mark.parametrize("mt,nt,k,ntot", [(4, 128, 512, 256), (2, 144, 512, 288), (1, 256, 64, 256)])
def test_tc_gemm_matches_float64(mt, nt, k, ntot):
    rng = np.random.default_rng(mt * 1000 + nt)
    M = mt * 128
    A = rng.uniform(-1, 1, (M, k)).astype(np.float32)
    B = (rng.standard_normal((k, ntot)) * 100).astype(np.float32)
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    dC = torch.zeros((M, ntot), dtype=torch.float32, device="cuda")
    xg.tc_gemm_check(mt, nt, k, ntot, dA.data_ptr(), dB.data_ptr(), dC.data_ptr())
    C = dC.cpu().numpy().astype(np.float64)
    ref = A.astype(np.float64) @ B.astype(np.float64)
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64)     # bound of the sum's magnitude
    err = np.abs(C - ref) / scale
    assert err.max() < 2e-6, (err.max(), np.unravel_index(err.argmax(), err.shape))
