"""Serving loop: jobs submitted while others run are admitted, coalesced into
batched sorts and overlapped across workers; every job's SA, BWT and primary
index must equal what the single-job path (the oracle) gives for it alone."""
import numpy as np
import pytest

import libsais_gb300 as G
from libsais_gb300 import textgen

pytestmark = pytest.mark.gpu


def make_jobs(rng, count):
    dna = textgen.markov2_dna(1 << 22, seed=11)
    zipf = textgen.zipf_u16(1 << 20, seed=12)
    jobs = []
    for k in range(count):
        u = rng.random()
        if k % 25 == 0:
            n = int(rng.integers(200_000, 1_000_000))      # a few large jobs (not coalesced)
        else:
            n = int(np.exp(rng.uniform(np.log(2), np.log(60_000))))
        if u < 0.7:
            a = int(rng.integers(0, dna.size - n))
            jobs.append(dna[a:a + n])
        elif u < 0.9:
            jobs.append(rng.integers(0, 256, n).astype(np.uint8))
        else:
            n = min(n, zipf.size - 1)
            a = int(rng.integers(0, zipf.size - n))
            jobs.append(zipf[a:a + n])
    return jobs


def test_server_results_match_single_job(oracle):
    rng = np.random.default_rng(41)
    jobs = make_jobs(rng, 150)
    srv = G.Server(hbm_budget_bytes=16 << 30, workers=2, small_job_symbols=1 << 16, max_batch=64)
    try:
        ids = [srv.submit(t) for t in jobs]
        assert all(i > 0 for i in ids)
        batched = 0
        for t, jid in zip(jobs, ids):
            res, SA, U, q, total, b = srv.wait(jid)
            p, oU, _, _ = oracle.libsais_bwt(t)
            _, oSA = oracle.sa(t)
            assert res == p, (t.size, res, p)
            assert np.array_equal(SA.astype(np.int64), oSA)
            assert np.array_equal(U, oU)
            assert total >= q >= 0
            batched += b > 1
        st = srv.stats()
        assert st["completed"] == st["submitted"] == len(jobs)
        assert st["batches"] > 0 and batched > 0            # small jobs were coalesced
        assert 0 < st["hbm_high_water_bytes"] <= st["hbm_budget_bytes"]
    finally:
        srv.close()


def test_server_coalesces_16bit_jobs(oracle):
    """Small 16-bit jobs are coalesced into batched sorts as 8-bit ones are."""
    rng = np.random.default_rng(43)
    zipf = textgen.zipf_u16(1 << 20, seed=13)
    jobs = []
    for _ in range(80):
        n = int(rng.integers(2, 20_000))
        a = int(rng.integers(0, zipf.size - n))
        jobs.append(zipf[a:a + n])
    srv = G.Server(hbm_budget_bytes=8 << 30, workers=1, small_job_symbols=1 << 15, max_batch=32)
    try:
        ids = [srv.submit(t) for t in jobs]
        batched = 0
        for t, jid in zip(jobs, ids):
            res, SA, U, q, total, b = srv.wait(jid)
            p, oU, _, _ = oracle.libsais_bwt(t)
            _, oSA = oracle.sa(t)
            assert res == p and np.array_equal(SA.astype(np.int64), oSA) and np.array_equal(U, oU)
            batched += b > 1
        assert batched > 0 and srv.stats()["batches"] > 0
    finally:
        srv.close()


def test_server_admits_against_one_pool(oracle):
    """A job larger than budget / workers but within the budget is admitted
    (one pool, not per-worker shares), and the pool's high-water mark stays
    within the budget while several such jobs queue."""
    budget = 512 << 20
    srv = G.Server(hbm_budget_bytes=budget, workers=3, small_job_symbols=1 << 10, max_batch=8)
    try:
        jobs = [textgen.genome_like(3 << 20, seed=50 + k) for k in range(4)]   # ~250 MiB footprint each
        ids = [srv.submit(t) for t in jobs]
        for t, jid in zip(jobs, ids):
            res, SA, U, *_ = srv.wait(jid)
            p, oU, _, _ = oracle.libsais_bwt(t)
            assert res == p and np.array_equal(U, oU)
        st = srv.stats()
        assert st["rejected"] == 0
        assert 0 < st["hbm_high_water_bytes"] <= budget
    finally:
        srv.close()


def test_server_rejects_job_over_budget():
    srv = G.Server(hbm_budget_bytes=64 << 20, workers=2, small_job_symbols=1 << 10, max_batch=8)
    try:
        big = textgen.iid(1 << 20, seed=3)       # 80 B/symbol footprint > the 64 MiB budget
        jid = srv.submit(big)
        res, *_ = srv.wait(jid)
        assert res == -2
        small = textgen.iid(1000, seed=4)
        res, SA, U, *_ = srv.wait(srv.submit(small))
        assert res > 0
        assert srv.stats()["rejected"] == 1
    finally:
        srv.close()
