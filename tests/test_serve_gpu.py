"""Continuous-batching server: requests admitted under an HBM budget while
others run, each result the same alone and in the mix."""
import threading
import time

import numpy as np
import pytest
import scipy.sparse as sp

import block_matrix_format_performance_gb300 as bm

pytestmark = pytest.mark.gpu

GRIDS = [(20, 5), (40, 10), (64, 16), (30, 8), (80, 20), (24, 6), (52, 13), (100, 25)]


@pytest.fixture(scope="module")
def problems(lib, cuda):
    out = []
    for nx, ny in GRIDS:
        rp, c, v, rhs = bm.gen_q4_elasticity(nx, ny)
        out.append((bm.Matrix.from_bcsr(rp, c, v, 2), rp, c, v, rhs))
    return out


def loads(n, seed):
    return np.random.default_rng(seed).uniform(-1, 1, n)


def rel_residual(rp, c, v, b, x):
    crp, cc, cv = bm.bcsr_to_csr(rp, c, v, 2)
    K = sp.csr_matrix((cv, cc, crp))
    return np.linalg.norm(b - K @ x) / np.linalg.norm(b)


def test_mix_equals_alone_bitwise(problems):
    mix = bm.Server("fp64", tol=1e-10, max_batch=3)
    reqs = []
    # submit from two threads with small gaps, so requests join while others run
    def producer(idx):
        for k in idx:
            m, rp, c, v, _ = problems[k % len(problems)]
            b = loads(m.rows, 100 + k)
            x = np.full(m.rows, np.nan)
            reqs.append((k, b, x, mix.submit(m, b, x)))
            time.sleep(0.0005)
    threads = [threading.Thread(target=producer, args=(range(i, 16, 2),)) for i in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    results = {k: (b, x, mix.wait(t)) for k, b, x, t in reqs}
    stats = mix.stats()
    assert stats["completed"] == 16 and stats["micro_batches"] >= 2 and stats["in_flight"] == 0
    mix.close()
    for k, (b, x, info) in sorted(results.items())[:8]:
        m, rp, c, v, _ = problems[k % len(problems)]
        assert info["status"] == bm.SUCCESS, info
        assert rel_residual(rp, c, v, b, x) < 1e-10
        alone = bm.Server("fp64", tol=1e-10)
        x1 = np.full(m.rows, np.nan)
        i1 = alone.wait(alone.submit(m, b, x1))
        alone.close()
        assert i1["iterations"] == info["iterations"]
        assert np.array_equal(x.view(np.uint64), x1.view(np.uint64)), k


def test_admission_respects_the_budget(problems):
    m, rp, c, v, _ = problems[4]  # 80x20 -> 3200 rows
    # b and x, and ten FP64 work vectors (r, rh, p, v, s, t, residual, best x,
    # snapshot, accumulated update), each slice 256-byte aligned
    per_request = 256 * 2 * ((m.rows * 8 + 255) // 256) + ((m.rows * 80 + 255) // 256) * 256
    srv = bm.Server("fp64", tol=1e-10, hbm_budget_bytes=int(2.5 * per_request))
    xs = [np.zeros(m.rows) for _ in range(6)]
    bs = [loads(m.rows, k) for k in range(6)]
    tickets = [srv.submit(m, b, x) for b, x in zip(bs, xs)]
    infos = [srv.wait(t) for t in tickets]
    st = srv.stats()
    srv.close()
    assert all(i["status"] == bm.SUCCESS for i in infos)
    assert st["peak_bytes"] <= int(2.5 * per_request)
    for b, x in zip(bs, xs):
        assert rel_residual(rp, c, v, b, x) < 1e-10


def test_request_larger_than_budget_is_refused(problems):
    m = problems[7][0]
    srv = bm.Server("fp64", hbm_budget_bytes=1024)
    with pytest.raises(bm.BmfpError) as e:
        srv.submit(m, np.ones(m.rows), np.zeros(m.rows))
    assert e.value.status == bm.ERROR_BUDGET
    srv.close()


def test_large_requests_take_the_whole_gpu_lane(problems):
    srv = bm.Server("fp64", tol=1e-10, wide_threshold_rows=3000)
    todo = []
    for k in (7, 0, 4, 1):  # 100x25 and 80x20 go wide, the others batch
        m, rp, c, v, _ = problems[k]
        b = loads(m.rows, k)
        x = np.zeros(m.rows)
        todo.append((rp, c, v, b, x, srv.submit(m, b, x)))
    for rp, c, v, b, x, t in todo:
        info = srv.wait(t)
        assert info["status"] == bm.SUCCESS and rel_residual(rp, c, v, b, x) < 1e-10
    st = srv.stats()
    srv.close()
    assert st["wide_solves"] == 2 and st["micro_batches"] >= 1


def test_mixed_precision_server(problems):
    srv = bm.Server("mixed", tol=1e-10)
    todo = []
    for k in (0, 1, 5):
        m, rp, c, v, _ = problems[k]
        b = loads(m.rows, k)
        x = np.zeros(m.rows)
        todo.append((rp, c, v, b, x, srv.submit(m, b, x)))
    for rp, c, v, b, x, t in todo:
        info = srv.wait(t)
        assert info["status"] == bm.SUCCESS and rel_residual(rp, c, v, b, x) < 1e-10
    srv.close()


def test_finished_request_leaves_before_its_micro_batch(problems):
    """One stream: a first request occupies it, the next four wait and are
    launched together (one slow 200x50 system, three 20x5). The small ones
    come back while the slow one of the same launch is still running."""
    rp, c, v, _ = bm.gen_q4_elasticity(200, 50)
    big = bm.Matrix.from_bcsr(rp, c, v, 2)
    srv = bm.Server("fp64", tol=1e-10, streams=1, max_batch=8)
    first = srv.submit(big, loads(big.rows, 1), np.zeros(big.rows))
    deadline = time.time() + 10
    while srv.stats()["pending"] and time.time() < deadline:  # launched alone
        time.sleep(1e-4)
    b_slow = loads(big.rows, 2)
    x_slow = np.zeros(big.rows)
    slow = srv.submit(big, b_slow, x_slow)
    small = []
    for k in range(3):
        m, rp0, c0, v0, _ = problems[0]
        b = loads(m.rows, 10 + k)
        x = np.zeros(m.rows)
        small.append((rp0, c0, v0, b, x, srv.submit(m, b, x)))
    srv.wait(first)
    early, slow_info = 0, None
    for rp0, c0, v0, b, x, t in small:
        info = srv.wait(t)
        assert info["status"] == bm.SUCCESS and rel_residual(rp0, c0, v0, b, x) < 1e-10
        if slow_info is None:
            slow_info = srv.poll(slow)
            early += slow_info is None
    if slow_info is None:
        slow_info = srv.wait(slow)
    assert slow_info["status"] == bm.SUCCESS and rel_residual(rp, c, v, b_slow, x_slow) < 1e-10
    st = srv.stats()
    srv.close()
    big.close()
    assert st["micro_batches"] == 2  # the first request, then the four together
    assert early == 3


def _diag_dominant(nbr, seed):
    rng = np.random.default_rng(seed)
    rows = [np.unique(np.concatenate([[i], rng.integers(max(0, i - 10), min(nbr, i + 11), 6)])) for i in range(nbr)]
    rp = np.concatenate([[0], np.cumsum([len(r) for r in rows])]).astype(np.int32)
    c = np.concatenate(rows).astype(np.int32)
    v = rng.uniform(-1, 1, c.size * 4)
    for i in range(nbr):
        k = rp[i] + int(np.where(rows[i] == i)[0][0])
        v[k * 4:(k + 1) * 4].reshape(2, 2)[...] += np.eye(2) * (len(rows[i]) * 3.0)
    return rp, c, v


def test_mixed_mix_equals_alone_bitwise(problems):
    """Mixed precision served: micro-batched requests (elasticity, whose FP32
    steps fail, and a well-conditioned matrix refined in FP32) and whole-GPU
    lane requests (the lane's solver decides FP32 or FP64 once, from the
    matrix) give the same bits alone as in a mix of 14 requests."""
    rp, c, v = _diag_dominant(1500, 3)
    good = (bm.Matrix.from_bcsr(rp, c, v, 2), rp, c, v, None)
    pool = [problems[0], problems[1], problems[4], problems[7], good]  # 80x20 and 100x25 go wide
    mix = bm.Server("mixed", tol=1e-10, max_batch=4, wide_threshold_rows=3000)
    reqs = []
    for k in range(14):
        m = pool[k % len(pool)][0]
        b = loads(m.rows, 300 + k)
        x = np.full(m.rows, np.nan)
        reqs.append((k, b, x, mix.submit(m, b, x)))
    results = [(k, b, x, mix.wait(t)) for k, b, x, t in reqs]
    st = mix.stats()
    mix.close()
    assert st["wide_solves"] >= 2 and st["micro_batches"] >= 1
    refined = 0
    for k, b, x, info in results[:len(pool)]:
        m, rp0, c0, v0, _ = pool[k % len(pool)]
        assert info["status"] == bm.SUCCESS and rel_residual(rp0, c0, v0, b, x) < 1e-10, info
        refined += info["iterations_fp32"] > 0 and not info["used_fp64_fallback"]
        alone = bm.Server("mixed", tol=1e-10, wide_threshold_rows=3000)
        x1 = np.full(m.rows, np.nan)
        i1 = alone.wait(alone.submit(m, b, x1))
        alone.close()
        for key in ("iterations", "iterations_fp32", "used_fp64_fallback"):
            assert i1[key] == info[key], (k, key, i1, info)
        assert np.array_equal(x.view(np.uint64), x1.view(np.uint64)), k
    assert refined >= 1
    good[0].close()
