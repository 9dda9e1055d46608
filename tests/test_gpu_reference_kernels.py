"""The reference's own GPU kernels (myhpu_extension_kernel.cu compiled
unmodified for sm_103a into oracle/_ref by oracle/build.py), launched by
oracle/ref_gpu.py as the reference's launchers do: its `--cuda` flow over them
reproduces the golden peel order recorded from the reference's drivers, and
its support kernel agrees with this build's.  These are the reference GPU path
bench.py times; skipped where the image was not built (no reference tree when
the repository was built)."""
import numpy as np
import pytest
import torch

from oracle import ref_gpu as RG
from tests import _golden as GD
from tdtdecomposition_gb300 import CSRCOO, truss as T

pytestmark = pytest.mark.gpu

if not RG.available():
    pytest.skip("reference kernel image not built", allow_module_level=True)


@pytest.fixture(scope="module")
def kernels():
    return RG.RefKernels()


def _cu(a, dtype=torch.int32):
    return torch.as_tensor(np.asarray(a), dtype=dtype).cuda()


@pytest.mark.parametrize("n_cut", [1, 2])
@pytest.mark.parametrize("name", ["fixture", "rmat_s10", "ba_1500_8"])
def test_reference_kernels_reproduce_the_golden_peel_order(kernels, name, n_cut):
    d = GD.load(name)
    V = d["ref_vertices"].shape[0]
    g = CSRCOO(columns=_cu(d["ref_cols"]), row_ptr=_cu(d["ref_rp_tiled%d" % n_cut]), rows=_cu(d["ref_rows"]))
    kmax, et, pt = RG.k_truss_on_reference_kernels(g, n_cut, V, kernels)
    assert kmax == int(d["sg_kmax%d" % n_cut])
    assert np.array_equal(et.cpu().numpy(), d["sg_e_truss%d" % n_cut])
    assert np.array_equal(pt.numpy(), d["sg_ptr_truss%d" % n_cut])


def test_reference_support_kernel_equals_ours(kernels):
    d = GD.load("er_4096_65536")
    rows, cols = _cu(d["ref_rows"]), _cu(d["ref_cols"])
    out = torch.zeros(cols.shape[0], dtype=torch.int32, device="cuda")
    kernels.segment_isin2tile(rows, cols, _cu(d["ref_rp_tiled2"]), 2, out)
    g = CSRCOO(columns=cols, row_ptr=_cu(d["ref_rp"], torch.int64), rows=rows)
    _, sup = T.triangle_count(g, return_support=True)
    assert torch.equal(out, sup)
    assert np.array_equal(out.cpu().numpy(), d["ref_support"])
