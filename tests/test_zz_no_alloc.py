"""The allocation-free stiffness apply (ems_tet_stiffness_apply_static) for
callers that cannot call cudaMalloc, checked through the C ABI against the
allocating entry point ems_tetfem_apply_stiffness on two calls in a row.
Both compute every curl term and every gather term in the same order with
the same FP32 operations (terms with a zero curl factor add an exact zero
in the allocation-free path and are skipped in the other), so their outputs
agree bit for bit.  Meshes: an ordinary one, a single cube (every slot PEC
except the cube's body diagonal) and the largest mesh the fixed scratch
holds.  The test owns the device buffers; the entry point itself allocates
nothing.  Collected last so a stop-at-first-failure run has executed every
other test before it."""
import ctypes as C

import numpy as np
import pytest

import emsolvers_gb300 as ems

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [(9, 8, 7), (1, 1, 1), (55, 55, 55)], ids=["9x8x7", "1x1x1", "55^3_max"])
def test_static_stiffness_apply_matches_allocating_entry_point_twice(n):
    torch = pytest.importorskip("torch")
    L = ems.lib()
    nslot = 7 * (n[0] + 1) * (n[1] + 1) * (n[2] + 1)
    rng = np.random.default_rng(42)
    sim = ems.TetFemSimulation(n, 1e-3, 1, ems.SYMP2, ems.FP32, dt=1e-13)
    cells = (C.c_int * 3)(*n)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        u = rng.standard_normal(nslot).astype(np.float32)
        f_ref = sim.apply_stiffness(u.astype(np.float64))
        u_d = torch.from_numpy(u).cuda()
        f_d = torch.full((nslot,), float("nan"), dtype=torch.float32, device="cuda")
        rc = L.ems_tet_stiffness_apply_static(cells, C.c_void_p(u_d.data_ptr()), C.c_void_p(f_d.data_ptr()), stream)
        assert rc == 0, L.ems_last_error(None)
        torch.cuda.synchronize()
        f = f_d.cpu().numpy().astype(np.float64)
        assert np.isfinite(f).all(), f"call {call}: output not fully written"
        assert np.abs(f_ref).max() > 0
        assert np.array_equal(f, f_ref), f"call {call}: differs from the allocating entry point"
    sim.close()


def test_static_stiffness_apply_rejects_meshes_beyond_its_scratch():
    L = ems.lib()
    cells = (C.c_int * 3)(64, 64, 64)   # 1,572,864 tetrahedra > 2^20
    rc = L.ems_tet_stiffness_apply_static(cells, C.c_void_p(16), C.c_void_p(16), None)
    assert rc == -1
    assert b"exceeds the fixed scratch" in L.ems_last_error(None)
