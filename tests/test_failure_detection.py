"""Failure detection, tested without faulting, trapping or hanging a GPU.

The reference has no failure handling (it panics on bad input, src/link.rs:19-21);
the GPU path adds two device-side checks, both reported through the device
error word as B2D_ERR_DEVICE at the next synchronisation:
* every bulk-copy wait of the link executor is bounded; a wait that gives up
  records the failure, waits for its copy in flight to land and leaves.  The
  B2D_FAULT_WAIT_TIMEOUT switch makes each group take that path on its first
  wait (the copy still completes normally), in the resident-schedule and the
  streamed-schedule executors;
* the collision grid refuses an entry that would land past its capacity
  instead of writing past it: an overflow entry of the slotted grid (a
  bucket's entries past its fixed slots), or a block of sorted entries of
  the sorted grid (larger grids, or tunable grid_slot_max = 0);
  B2D_FAULT_GRID_CAP lowers the capacity the kernels see.
After each failure the solver state is rewritten and the next update must
match the oracle bit for bit: the context stays usable.  Host-side
failures (an allocation that fails) are injected on the host."""
import numpy as np
import pytest

from helpers import assert_same_state, oracle_state, solver_state

pytestmark = pytest.mark.gpu


def _grids(collide, seed=3, n_bodies=6, clump=False):
    """Cloth grids; with clump, also a 3 x 3 grid packed into one collision
    cell (nine entries in one bucket: five past its fixed slots)."""
    from bendy2d_gb300 import scenes
    rng = np.random.default_rng(seed)
    bodies = [scenes.grid_body(32, 32, rng.uniform(0.0, 168.0, 2), 1.0, 0.01, rng)
              for _ in range(n_bodies)]
    if clump:
        bodies.append(scenes.grid_body(3, 3, (190.3, 190.3), 0.05, 0.0, rng))
    sc = scenes._assemble("grids", bodies, bounds=(0.0, 0.0, 200.0, 200.0), sub_steps=4,
                          link_iters=2, collide=collide)
    sc.prev = scenes._velocity_prev(sc.pos, rng, 0.5, sc.dt / sc.sub_steps)
    return sc


def _fail_then_recover(sc, kind, value, tuning=None, expect="bulk-copy wait", warm=True):
    """One good update (warm), one update under the fault (B2D_ERR_DEVICE),
    then the state before it is written back and one more update must equal
    the oracle's next update."""
    from bendy2d_gb300 import B2DError
    from oracle import load_scene
    s = sc.to_solver()
    if tuning:
        s.set_tuning(**tuning)
    o = load_scene(sc)
    if warm:
        s.update(sc.dt)
        assert o.update(sc.dt) == 0
        assert_same_state(solver_state(s), oracle_state(o), "before the fault")
    pos0, prev0 = s.read_state()
    s.set_fault(kind, value)
    with pytest.raises(B2DError) as e:
        s.update(sc.dt)
        s.synchronize()
    assert e.value.code == 8, e.value
    assert expect in str(e.value)
    s.set_fault(kind, 0)
    s.write_state(pos0, prev0)
    s.update(sc.dt)
    assert o.update(sc.dt) == 0
    assert_same_state(solver_state(s), oracle_state(o), "after recovery")
    s.close()


@pytest.mark.parametrize("collide", [0, 1])
@pytest.mark.parametrize("resident", [0, 1])
def test_bulk_copy_wait_timeout_is_reported_and_recovered(gpu, collide, resident):
    from bendy2d_gb300._native import FAULT_WAIT_TIMEOUT
    sc = _grids(collide)
    _fail_then_recover(sc, FAULT_WAIT_TIMEOUT, 1, tuning={"resident": resident})


@pytest.mark.parametrize("sorted_grid", [0, 1])
def test_grid_capacity_overflow_is_refused_and_recovered(gpu, sorted_grid):
    """Slotted grid: one overflow entry allowed against the clump's five (in
    the first sub-step, before the clump spreads).  Sorted grid: a quarter
    of the entries."""
    from bendy2d_gb300._native import FAULT_GRID_CAP
    sc = _grids(1, seed=5, clump=True)
    _fail_then_recover(sc, FAULT_GRID_CAP, sc.n_particles // 4 if sorted_grid else 1,
                       tuning={"grid_slot_max": 0 if sorted_grid else 1 << 30},
                       expect="grid entries past their capacity", warm=False)


@pytest.mark.parametrize("sorted_grid", [0, 1])
def test_grid_capacity_at_the_particle_count_is_not_an_error(gpu, sorted_grid):
    """A capacity equal to the particle count holds every entry: no error,
    results exact."""
    from bendy2d_gb300._native import FAULT_GRID_CAP
    from oracle import load_scene
    sc = _grids(1, seed=6, clump=True)
    s = sc.to_solver()
    s.set_tuning(grid_slot_max=0 if sorted_grid else 1 << 30)
    s.set_fault(FAULT_GRID_CAP, sc.n_particles)
    o = load_scene(sc)
    for _ in range(2):
        s.update(sc.dt)
        assert o.update(sc.dt) == 0
    s.synchronize()
    assert_same_state(solver_state(s), oracle_state(o), "capacity = particle count")


def test_injected_allocation_failure_leaves_the_solver_usable(gpu):
    """The world's device block fails to allocate at placement: the update
    reports B2D_ERR_CUDA and changes nothing; the next update places the
    world and matches the oracle."""
    from bendy2d_gb300 import B2DError
    from bendy2d_gb300._native import FAULT_ALLOC
    from oracle import load_scene
    sc = _grids(1, seed=7, n_bodies=2)
    s = sc.to_solver()
    s.set_fault(FAULT_ALLOC, 1)
    with pytest.raises(B2DError) as e:
        s.update(sc.dt)
    assert e.value.code == 7 and "injected" in str(e.value)
    o = load_scene(sc)
    for _ in range(2):
        s.update(sc.dt)
        assert o.update(sc.dt) == 0
    assert_same_state(solver_state(s), oracle_state(o), "after a failed placement")


def test_unknown_fault_kind_is_rejected(gpu):
    from bendy2d_gb300 import B2DError, Solver
    s = Solver()
    with pytest.raises(B2DError) as e:
        s.set_fault(99, 1)
    assert e.value.code == 5
