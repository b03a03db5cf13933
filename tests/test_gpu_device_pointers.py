"""cutc_int_ex with device-resident inputs/outputs on a caller stream, both forms.

The device-pointer path must give the same bits as the host-pointer path (the
same kernels run on the same data), and fill the timing statistics.
"""
import numpy as np
import pytest

import cutc_gb300 as cg
from cutc_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [cg.PLAIN_FP64, cg.SPLIT_BF16])
def test_device_pointers_match_host_pointers(prec):
    import torch
    p = synth.make_problem(n_nuc=3, n_ao=11, n_grid1=333, n_grid2=1500, size_bh=7, seed=13)
    Xh, Ih = cg.build_integrals(p, prec, x_components=4)
    dev = torch.device("cuda", 0)
    dr = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in p.arrays().items()}
    Xd = torch.full((4, p.n_grid1, p.n_ao ** 2), float("nan"), dtype=torch.float64, device=dev)
    Id = torch.full((p.n_ao ** 2, p.n_ao ** 2), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    opt = cg.options(prec, None, p.a_en, p.a_ee, 4, True, 0, stream.cuda_stream)
    st = cg.Stats()
    s = cg.cutc_int_ex(opt, p.n_grid1, p.n_grid2, p.n_ao, p.n_nuc, p.size_bh,
                       dr["r1"], dr["wr1"], dr["r2"], dr["wr2"], dr["rn"], dr["aos1"], dr["aos2"],
                       dr["c_bh"], dr["m_bh"], dr["n_bh"], dr["o_bh"], Xd, Id, st)
    assert s == 0, cg.last_error()
    stream.synchronize()
    assert np.array_equal(Xd.cpu().numpy(), Xh)
    assert np.array_equal(Id.cpu().numpy(), Ih)
    assert st.gpu_launches > 0 and st.n_x_gemm == st.n_r1_tiles >= 1
    assert 0.0 < st.ms_x_gemm <= st.ms_total
