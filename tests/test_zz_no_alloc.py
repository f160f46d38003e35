"""b2d_collide_substeps_noalloc against b2d_update, through the C ABI.

The no-allocation entry point serves callers that may not allocate GPU
memory while they run (frame loops that reserve all device memory at
start-up, hosts that own every device buffer): it works on the caller's
device arrays and keeps its scratch in one static device array, which caps
it at 65536 particles.  Its results must equal, bit for bit, what
b2d_update computes for a solver holding the same link-free particles with
particle-particle collisions on — the same tolerance as every other parity
test here.  Two calls in a row check that the shared scratch array carries
nothing over from one call to the next.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scene(n, box, seed):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(1.0, box - 1.0, size=(n, 2)).astype(np.float32)
    vel = rng.normal(0.0, 2.0, size=(n, 2))
    prev = (pos - vel * (1.0 / 60.0) / 3).astype(np.float32)
    return pos, prev


def _params(N, box, sub_steps=3, cell=1.0):
    return N.CNoAllocParams(gravity_x=0.0, gravity_y=-9.81, bounds_x=0.0, bounds_y=0.0,
                            bounds_w=box, bounds_h=box, dt=1.0 / 60.0, sub_steps=sub_steps,
                            particle_radius=0.5, grid_cell=cell)


N = None


@pytest.fixture(scope="module")
def lib(gpu):
    global N
    from bendy2d_gb300 import _native
    N = _native
    return gpu


# odd sub-step counts end in the scratch position buffer (copied back), even
# ones in the caller's; a cell of 1.25 takes the division path of the cell
# coordinate, a power of two the exact reciprocal
@pytest.mark.parametrize("n,box,seed,sub,cell", [(5000, 60.0, 1, 3, 1.0), (40000, 100.0, 2, 3, 1.0),
                                                 (65536, 180.0, 3, 3, 1.0), (20000, 90.0, 4, 2, 1.0),
                                                 (30000, 110.0, 5, 3, 1.25)])
def test_noalloc_matches_update(lib, n, box, seed, sub, cell):
    import torch
    from bendy2d_gb300 import Bounds, Solver
    pos, prev = _scene(n, box, seed)
    # existing entry point: a solver holding the same particles
    s = Solver()
    s.gravity = (0.0, -9.81)
    s.bounds = Bounds((0.0, 0.0), (box, box))
    s.set_sub_steps(sub)
    s.set_collision(1, 0.5, cell)
    s.add_particles(pos, prev)
    # no-allocation entry point on caller-owned device arrays
    d_pos = torch.from_numpy(pos.copy()).cuda()
    d_prev = torch.from_numpy(prev.copy()).cuda()
    stream = torch.cuda.current_stream()
    prm = _params(N, box, sub, cell)
    for call in range(2):
        s.update(1.0 / 60.0)
        code = lib.b2d_collide_substeps_noalloc(C.c_void_p(d_pos.data_ptr()),
                                                C.c_void_p(d_prev.data_ptr()), n, C.byref(prm),
                                                C.c_void_p(stream.cuda_stream))
        assert code == 0, lib.b2d_last_error()
        torch.cuda.synchronize()
        ref_pos, ref_prev = s.read_state()
        got_pos, got_prev = d_pos.cpu().numpy(), d_prev.cpu().numpy()
        assert np.array_equal(got_pos.view(np.uint32), ref_pos.view(np.uint32)), \
            f"call {call}: positions differ (max {np.max(np.abs(got_pos - ref_pos)):.3g})"
        assert np.array_equal(got_prev.view(np.uint32), ref_prev.view(np.uint32)), \
            f"call {call}: previous positions differ"
    s.close()


def test_noalloc_rejects_too_many_particles(lib):
    prm = _params(N, 100.0)
    code = lib.b2d_collide_substeps_noalloc(C.c_void_p(1), C.c_void_p(1), 65537, C.byref(prm),
                                            None)
    assert code == 10
    assert b"at most 65536" in lib.b2d_last_error()
