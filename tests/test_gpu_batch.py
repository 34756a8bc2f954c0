"""Batched conversion (lm_batch_*): every job of a mixed batch, bit-exact
against the oracle, with and without CUDA-graph replay."""
import numpy as np
import pytest

from oracle import lm_oracle as O

pytestmark = pytest.mark.gpu


def oracle_of(op, src, d):
    from libmarshal_gb300 import lm
    if op == lm.OP_0100:
        return O.t0100(src, *d[:4])
    if op == lm.OP_010:
        return O.t010(src, *d[:3])
    if op == lm.OP_100:
        return O.t100(src, *d[:3])
    if op == lm.OP_AOS_ASTA:
        return O.aos_asta(src, *d[:3])
    if op == lm.OP_ASTA_AOS:
        h, w, t = d[:3]
        return O.t010(src, h // t, w, t)
    if op == lm.OP_SOA_ASTA:
        return O.soa_asta(src, *d[:3])
    if op == lm.OP_ASTA_SOA:
        h, w, t = d[:3]
        return O.t100(src, h // t, w, t)
    if op == lm.OP_TRANSPOSE:
        return O.transpose(src, *d[:2])
    raise ValueError(op)


def make_jobs(seed, n, lo, hi, big=()):
    from libmarshal_gb300 import lm
    rng = np.random.default_rng(seed)
    specs = []
    for k in range(n):
        e = int(rng.choice([1, 2, 4, 8]))
        h = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        w = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        kind = int(rng.integers(0, 8))
        t = int(rng.choice([16, 32, 64]))
        if kind == 0:
            op, d = lm.OP_TRANSPOSE, (h, w)
        elif kind == 1:
            op, d = lm.OP_AOS_ASTA, ((h + t - 1) // t * t, w, t)
        elif kind == 2:
            op, d = lm.OP_ASTA_AOS, ((h + t - 1) // t * t, w, t)
        elif kind == 3:
            op, d = lm.OP_SOA_ASTA, ((h + t - 1) // t * t, w, t)
        elif kind == 4:
            op, d = lm.OP_ASTA_SOA, ((h + t - 1) // t * t, w, t)
        elif kind == 5:
            op, d = lm.OP_100, (h, w, int(rng.choice([1, 2, 3])))
        elif kind == 6:
            op, d = lm.OP_010, (max(1, h // 16), 16, w)
        else:
            op, d = lm.OP_0100, (2, max(1, h // 8), w // 4 + 1, 3)
        specs.append((op, d, e))
    specs += list(big)
    return specs


def nelems(op, d):
    from libmarshal_gb300 import lm
    if op == lm.OP_0100:
        return d[0] * d[1] * d[2] * d[3]
    if op in (lm.OP_010, lm.OP_100):
        return d[0] * d[1] * d[2]
    if op == lm.OP_TRANSPOSE:
        return d[0] * d[1]
    return d[0] * d[1]


def run_and_check(cuda, specs, graph, reps, **flags):
    import torch
    from libmarshal_gb300 import lm
    srcs, bufs, jobs = [], [], []
    for k, (op, d, e) in enumerate(specs):
        n = nelems(op, d)
        src = O.random_bits(n, e, 1000 + k)
        srcs.append(src)
        b = torch.from_numpy(src.view(np.uint8).copy()).to(cuda)
        bufs.append(b)
        jobs.append(lm.job(b, op, d, elem_bytes=e))
    want = [oracle_of(op, s, d) for (op, d, e), s in zip(specs, srcs)]
    bt = lm.Batch()
    for rep in range(reps):
        if rep:
            for b, s in zip(bufs, srcs):  # same buffers, original data
                b.copy_(torch.from_numpy(s.view(np.uint8).copy()).to(cuda))
        bt.run(jobs, graph=graph, **flags)
        torch.cuda.synchronize()
        for k, ((op, d, e), b) in enumerate(zip(specs, bufs)):
            got = b.cpu().numpy().view(O.DTYPES[e])
            assert np.array_equal(got, want[k]), (rep, k, op, d, e)
    st = bt.stats()
    bt.close()
    assert lm.lib().lm_device_status(None) == 0
    return st


def test_batch_small_mixed(cuda):
    from libmarshal_gb300 import lm
    specs = make_jobs(1, 300, 16, 300)
    st = run_and_check(cuda, specs, graph=False, reps=1)
    assert st["small_jobs"] > 0


BIG = [(7, (2048, 1031), 4), (3, (4096, 3000, 64), 8), (7, (1500, 1700), 2),
       (2, (4096, 1000, 1), 1), (5, (1 << 16, 4, 32), 4),
       (0, (3, 1100, 700, 3), 2), (2, (2000, 1500, 2), 8)]


def test_batch_with_large_jobs_and_graph(cuda):
    specs = make_jobs(2, 120, 16, 1200, big=BIG)
    st = run_and_check(cuda, specs, graph=True, reps=3)
    assert st["staged_jobs"] > 0 and (st["small_jobs"] + st["big_jobs"]) > 0


def test_batch_strictly_in_place(cuda):
    """LM_BATCH_NO_SCRATCH: large jobs go through the in-place planner."""
    specs = make_jobs(4, 60, 16, 1200, big=BIG)
    st = run_and_check(cuda, specs, graph=True, reps=3, scratch=False)
    assert st["staged_jobs"] == 0 and st["large_jobs"] > 0


def test_batch_staged_waves(cuda, monkeypatch):
    """A small arena: several waves, jobs above it fall back to the planner."""
    monkeypatch.setenv("LM_BATCH_SCRATCH_MB", "9")
    specs = make_jobs(5, 60, 16, 1200, big=BIG + [(7, (777, 2999), 1)] * 3)
    st = run_and_check(cuda, specs, graph=True, reps=3)
    assert st["staged_waves"] > 1 and st["large_jobs"] > 0


def test_batch_rejects_bad_jobs(cuda):
    import torch
    from libmarshal_gb300 import lm
    b = torch.zeros(64, dtype=torch.uint8, device=cuda)
    bt = lm.Batch()
    with pytest.raises(lm.LMError):
        bt.run([lm.job(b, lm.OP_AOS_ASTA, (10, 3, 4), elem_bytes=1)])
    with pytest.raises(lm.LMError):
        bt.run([lm.job(b, lm.OP_TRANSPOSE, (8, 8), elem_bytes=3)])
    bt.run([lm.job(b, lm.OP_TRANSPOSE, (1, 64), elem_bytes=1)])  # identity
    bt.close()


# Tiles too large for one CTA's shared memory tile budget (40 KB) but small
# enough for a cluster of 2..16 CTAs (two stages of column bands of at most
# ~109 KB each), with odd, unaligned row lengths and every element width.
BAND_SPECS = [
    (7, (256, 300), 4),                 # clusters of 8, two CTAs per SM
    (7, (333, 777), 2),                 # unaligned rows
    (3, (64 * 7, 3000, 64), 8),         # 7 tiles of 64 x 3000, clusters of 16
    (2, (500, 999, 3), 1),              # b = 3, bytes
    (7, (600, 350), 4),
    (7, (1000, 300), 4),                # 1000 rows
    (0, (5, 100, 2000, 1), 4),          # 5 tiles
    (0, (3, 200, 150, 5), 8),           # b = 5, 8-byte elements
    (4, (64 * 5, 1000, 64), 8),         # ASTA -> AoS, 1000-row tiles
]


@pytest.mark.parametrize("graph,scratch", [(False, False), (True, False),
                                           (True, True)])
def test_batch_cluster_items(cuda, graph, scratch):
    specs = make_jobs(3, 40, 16, 200, big=BAND_SPECS)
    st = run_and_check(cuda, specs, graph=graph, reps=3 if graph else 1,
                       scratch=scratch)
    if not scratch:  # every cluster size, one and two CTAs per SM
        assert st["band_jobs"] >= len(BAND_SPECS), st
    assert st["band_items"] >= st["band_jobs"] > 0


def test_batch_cluster_off_matches(cuda):
    """LM_BATCH_NO_CLUSTER sends the same jobs through the per-op planner."""
    import torch
    from libmarshal_gb300 import lm
    srcs, outs = [], []
    for cluster in (True, False):
        bufs, jobs = [], []
        for k, (op, d, e) in enumerate(BAND_SPECS):
            src = O.random_bits(nelems(op, d), e, 77 + k)
            b = torch.from_numpy(src.view(np.uint8).copy()).to(cuda)
            bufs.append(b)
            jobs.append(lm.job(b, op, d, elem_bytes=e))
        bt = lm.Batch()
        bt.run(jobs, cluster=cluster)
        torch.cuda.synchronize()
        st = bt.stats()
        bt.close()
        assert (st["band_jobs"] > 0) == cluster
        outs.append([b.cpu().numpy() for b in bufs])
    for x, y in zip(*outs):
        assert np.array_equal(x, y)


def test_batch_vector_tile_items(cuda):
    """AoS->ASTA jobs on 16-byte aligned buffers whose output rows are whole
    16-byte vectors: tiles up to 16 KB (several per item) and of 16-112 KB
    (one per item) run through the batched 16-byte tile kernel, beside jobs
    it does not take (ASTA->AoS, odd tiles), with and without graph
    replay; every result against the oracle."""
    from libmarshal_gb300 import lm
    specs = []
    for k, (h, w, t, e) in enumerate([
            (64 * 30, 11, 64, 1), (32 * 50, 7, 32, 4), (16 * 40, 200, 16, 8),
            (64 * 9, 700, 64, 1), (32 * 8, 1000, 32, 2), (16 * 6, 900, 16, 8),
            (32 * 100, 3, 32, 2), (64 * 3, 1700, 64, 1)]):
        specs.append((lm.OP_AOS_ASTA, (h, w, t), e))
        specs.append((lm.OP_ASTA_AOS, (h, w, t), e))
    specs.append((lm.OP_010, (40, 12, 5), 1))
    lm.prof_collect()
    lm.prof_enable(True)
    try:
        st = run_and_check(cuda, specs, graph=False, reps=1)
        run_and_check(cuda, specs, graph=True, reps=3)
    finally:
        lm.prof_enable(False)
    ran = lm.prof_collect()
    # form A (AoS->ASTA: whole-vector output rows) and form B (ASTA->AoS
    # specs such as 11 x 64 bytes, 7 x 32 x 4 and 3 x 32 x 2: whole-vector
    # input rows) both ran
    assert "batch_tile010" in ran, ran
    assert "batch_tile010b" in ran, ran
    assert st["small_jobs"] > 0


def test_batch_full_4096_matrix_list(cuda):
    """The batched configuration at its full size: the 4096 matrices of seed
    1 (sides log-uniform in [16, 4096], widths 1/2/4/8 bytes, AoS->ASTA with
    tiles 16/32/64 or the full transpose; 9.4 GB) in one arena, converted by
    one batch call and by a CUDA-graph replay of the same list, every job
    compared with the oracle each time."""
    import torch
    import bench
    from libmarshal_gb300 import lm
    from oracle import check as C
    specs = bench.batch_specs(n=4096)
    offs, tot = [], 0
    vjobs = []
    for op, d, e in specs:
        code = C.OP_AOS_ASTA if op == "aos_asta" else C.OP_TRANSPOSE
        offs.append(tot)
        vjobs.append((tot, code, d, e))
        tot += (C.n_elems(code, d) * e + 255) // 256 * 256
    arena = torch.empty(tot, dtype=torch.uint8, device=cuda)
    base = arena.data_ptr()
    jobs = [lm.Job(base + off, e, code, *(list(d) + [0] * (4 - len(d))))
            for (off, code, d, e) in vjobs]
    bt = lm.Batch()

    def fill_run_check(graph):
        host = np.empty(tot, dtype=np.uint8)
        C.fill_host(host, vjobs, 4 << 20)
        arena.copy_(torch.from_numpy(host))
        del host
        bt.run(jobs, graph=graph)
        torch.cuda.synchronize()
        bad = C.check_host(arena.cpu().numpy(), vjobs, 4 << 20)
        assert not bad, ("graph" if graph else "batched", bad[:10])

    fill_run_check(False)
    bt.run(jobs, graph=True)  # first run of the list with graphs on
    bt.run(jobs, graph=True)  # second: captured into a graph
    fill_run_check(True)      # later runs replay it
    bt.close()
    assert lm.lib().lm_device_status(None) == 0
    del arena
    torch.cuda.empty_cache()


def test_batch_tuned_variants(cuda):
    """The autotuner's variants (the planner's choice; the staged form with
    16, 32 or 64 KB blocks; whole-cycle moves; the stash plan with the
    planner's, one or two CTAs per SM; the two-pass split; cycle following)
    each pinned for its shape class with lm_tune_variant and run through the
    batch executor's tuned path (jobs of 16 MB or more), bit-exact against
    the oracle; a variant that does not apply to the shape falls back to the
    planner.  Then a class with no entry is tuned by timing."""
    from libmarshal_gb300 import lm
    lib = lm.lib()
    shapes = [  # (op, dims, e): staged-form, stash-plan, short-cycle shapes
        (lm.OP_TRANSPOSE, (3000, 2000), 4),
        (lm.OP_100, (8000, 600, 1), 4),
        (lm.OP_SOA_ASTA, (131072 * 32, 4, 32), 4),
    ]
    for op, d, e in shapes:
        if op == lm.OP_TRANSPOSE:
            T, a, B, b = 1, d[0], d[1], 1
        elif op == lm.OP_100:
            T, a, B, b = 1, d[0], d[1], d[2]
        else:  # SoA -> ASTA: 100(w, h / t, t)
            T, a, B, b = 1, d[1], d[0] // d[2], d[2]
        for v in range(10):
            assert lib.lm_tune_variant(e, T, a, B, b, v) == v
            run_and_check(cuda, [(op, d, e)], graph=False, reps=1)
    # an untuned class (2-byte 9000 x 1100 transposition) gets an entry
    T, a, B, b = 1, 9000, 1100, 1
    n0 = lib.lm_tune_entries()
    assert lib.lm_tune_variant(2, T, a, B, b, -1) == -1
    run_and_check(cuda, [(lm.OP_TRANSPOSE, (a, B), 2)], graph=False, reps=1)
    assert lib.lm_tune_variant(2, T, a, B, b, -1) >= 0
    assert lib.lm_tune_entries() == n0 + 1
