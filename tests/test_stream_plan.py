"""The streamed render's bookkeeping, restated on the CPU (no GPU): the host fixes the iteration
count of `issue_stream` and the radiance ring's size (`stream_ring_entries`) before any kernel
runs, so that the launch sequence can be captured in a graph. These tests check that those bounds
suffice for the plan / refill / shade rules of `k_stream_plan`, `k_regen` and `shade_queue<true>`
(csrc/tt_render_native.cu), on random path lengths:

- every path ends by the final plan (the device would otherwise flag kErrStream);
- no ring entry is overwritten before its path was accumulated;
- paths are accumulated exactly once and in index order (so images equal the wave scheme's);
- the queue never holds more than the pool.
"""
import numpy as np
import pytest

K_MAX_RING_ENTRIES = 1 << 29  # stream_ring_entries: beyond this a render runs in waves


def ring_entries(pool: int, max_depth: int) -> int:
    n = pool * max_depth
    return n if n <= K_MAX_RING_ENTRIES else 0


def iterations(total: int, pool: int, max_depth: int) -> int:
    """issue_stream's bound: every iteration extends a full pool while paths remain, then the
    pool drains in max_depth more."""
    return -(-total // pool) * max_depth + max_depth


def run(total: int, pool: int, max_depth: int, life: np.ndarray, iters: int | None = None) -> dict:
    """One streamed render of `total` paths; life[g] = bounces path g takes (1 .. max_depth).
    Returns the accumulation order and whether the final plan found every path ended."""
    ring_n = ring_entries(pool, max_depth)
    assert ring_n > 0
    iters = iterations(total, pool, max_depth) if iters is None else iters
    nxt, frontier, min_alive = 0, 0, None
    queue: list[int] = []  # path indices in queue order (state kept in queue order)
    depth: dict[int, int] = {}
    ring_owner: dict[int, int] = {}
    accumulated: list[int] = []
    err_stream = False
    ring_waits = 0  # plans whose refill the ring's room cut below the free slots and paths left
    for it in range(iters + 1):
        final = it == iters
        # k_stream_plan
        alive = len(queue)
        front = nxt if min_alive is None or min_alive >= nxt else min_alive
        for g in range(frontier, front):  # k_accumulate_stream: [acc_lo, acc_hi)
            assert ring_owner.get(g % ring_n) == g, "ring entry overwritten before accumulation"
            accumulated.append(g)
        frontier = front
        n_new = 0
        if not final:
            room = front + ring_n - nxt
            ring_waits += room < min(pool - alive, total - nxt)
            n_new = max(0, min(pool - alive, total - nxt, room))
        elif front != total:
            err_stream = True
        # k_regen: new paths behind the survivors
        for t in range(n_new):
            g = nxt + t
            depth[g] = 0
            queue.append(g)
        nxt += n_new
        min_alive = None
        assert len(queue) <= pool
        if final:
            break
        # extend + shade_queue<true>: survivors keep their order in the next queue, ended paths
        # leave their radiance in the ring, survivors report the smallest index among them
        survivors = []
        for g in queue:
            depth[g] += 1
            if depth[g] < life[g]:
                survivors.append(g)
                min_alive = g if min_alive is None else min(min_alive, g)
            else:
                slot = g % ring_n
                assert slot not in ring_owner or ring_owner[slot] < frontier, "ring slot still pending"
                ring_owner[slot] = g
        queue = survivors
    return {"accumulated": accumulated, "err_stream": err_stream, "ring_waits": ring_waits}


CASES = [(1000, 100, 8), (1000, 100, 1), (12345, 1000, 3), (5000, 4999, 8), (100_000, 4096, 16), (7, 3, 2),
         (4096, 4096, 8), (4097, 4096, 8)]


@pytest.mark.parametrize("total,pool,max_depth", CASES)
@pytest.mark.parametrize("p_continue", [0.0, 0.6, 0.95, 1.0])
def test_every_path_is_accumulated_once_in_order(total, pool, max_depth, p_continue):
    rng = np.random.default_rng(total + pool + max_depth)
    if p_continue >= 1.0:
        life = np.full(total, max_depth)  # every path runs to the depth limit
    else:
        life = np.minimum(rng.geometric(1.0 - p_continue, total), max_depth)
    r = run(total, pool, max_depth, life)
    assert not r["err_stream"]
    assert r["accumulated"] == list(range(total))
    assert r["ring_waits"] == 0


@pytest.mark.parametrize("seed", range(200))
def test_the_bound_holds_without_its_drain_term(seed):
    """The host's bound adds max_depth drain iterations to ceil(paths / pool) * max_depth, but the
    refill rules already finish by then: path g starts by the plan of iteration
    floor(g / pool) * max_depth (every earlier generation of pool paths has ended by then, which
    leaves free slots and ring room for it) and ends within max_depth iterations. So the last
    max_depth iterations of the bound only ever find empty queues."""
    rng = np.random.default_rng(seed)
    pool, max_depth, total = int(rng.integers(1, 12)), int(rng.integers(1, 9)), int(rng.integers(1, 120))
    kind = seed % 3
    if kind == 0:
        life = rng.integers(1, max_depth + 1, total)
    elif kind == 1:
        life = np.where(rng.random(total) < 0.1, max_depth, 1)  # stragglers among short paths
    else:
        life = np.where(rng.random(total) < 0.7, max_depth, rng.integers(1, max_depth + 1, total))
    short = iterations(total, pool, max_depth) - max_depth
    r = run(total, pool, max_depth, life, iters=short)
    assert not r["err_stream"] and r["accumulated"] == list(range(total))
    assert r["ring_waits"] == 0


def test_a_bound_below_that_leaves_paths_unfinished():
    """Paths that all run to the depth limit fill the pool generation by generation, so one
    iteration fewer than ceil(paths / pool) * max_depth leaves the last generation running: the
    final plan flags the render (kErrStream) and what it accumulated is a prefix, in order."""
    total, pool, max_depth = 1000, 100, 8
    life = np.full(total, max_depth)
    r = run(total, pool, max_depth, life, iters=iterations(total, pool, max_depth) - max_depth - 1)
    assert r["err_stream"]
    assert r["accumulated"] == list(range(len(r["accumulated"]))) and len(r["accumulated"]) < total


def test_one_straggler_holds_the_frontier_but_not_the_refill():
    """A path that runs to the depth limit while all later ones end at once holds the frontier
    (the accumulation) back for max_depth iterations. The ring's pool x max_depth entries hold
    every path that ends meanwhile, so the refill never waits for room: the straggler started at
    most max_depth iterations ago, and at most a pool of paths start per iteration."""
    total, pool, max_depth = 2000, 16, 8
    life = np.ones(total, dtype=int)
    life[3] = max_depth
    r = run(total, pool, max_depth, life)
    assert not r["err_stream"] and r["accumulated"] == list(range(total))
    assert r["ring_waits"] == 0


def test_large_pools_fall_back_to_waves():
    assert ring_entries(1 << 26, 8) == 1 << 29
    assert ring_entries(1 << 26, 16) == 0
