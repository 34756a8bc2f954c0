"""Conversion server (lm_serve_*): every request bit-exact against the oracle,
alone and in a continuously batched mix, on device buffers and staged from
host memory under a small HBM budget."""
import threading
import time

import numpy as np
import pytest

from oracle import lm_oracle as O
from test_gpu_batch import make_jobs, nelems, oracle_of

pytestmark = pytest.mark.gpu


def _device_reqs(cuda, specs, seed0):
    import torch
    srcs, bufs = [], []
    for k, (op, d, e) in enumerate(specs):
        src = O.random_bits(nelems(op, d), e, seed0 + k)
        srcs.append(src)
        bufs.append(torch.from_numpy(src.view(np.uint8).copy()).to(cuda))
    return srcs, bufs


def _check(specs, srcs, outs):
    for k, ((op, d, e), s, got) in enumerate(zip(specs, srcs, outs)):
        want = oracle_of(op, s, d)
        assert np.array_equal(got.view(O.DTYPES[e]), want), (k, op, d, e)


def test_serve_device_mix_matches_alone(cuda):
    """Each result is identical when served alone and in the mix."""
    import torch
    from libmarshal_gb300 import lm
    big = [(7, (1500, 1700), 2), (3, (4096, 3000, 64), 8),
           (2, (9000, 1000, 1), 8)]  # the last one is above 64 MiB
    specs = make_jobs(11, 150, 16, 900, big=big)
    srcs, bufs = _device_reqs(cuda, specs, 500)
    torch.cuda.synchronize()
    srv = lm.Server(8 << 30)
    tickets = [srv.submit(op, d, e, buf=b) for (op, d, e), b in zip(specs, bufs)]
    srv.drain(60000)
    done = {t: (st, lat) for t, st, lat, _ in srv.poll(10000)}
    assert sorted(done) == sorted(tickets)
    assert all(st == 0 and lat > 0 for st, lat in done.values())
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(specs) and st["batches"] >= 1
    _check(specs, srcs, [b.cpu().numpy() for b in bufs])
    # alone: a fresh server per request, on a few of them
    for k in (0, len(specs) // 2, len(specs) - 1):
        op, d, e = specs[k]
        b = torch.from_numpy(srcs[k].view(np.uint8).copy()).to(cuda)
        one = lm.Server(8 << 30)
        one.submit(op, d, e, buf=b)
        one.drain(60000)
        one.close()
        assert np.array_equal(b.cpu().numpy(), bufs[k].cpu().numpy())


def test_serve_host_staging_under_budget(cuda):
    """Host requests through a pool smaller than their sum: admission makes
    them wait, every result comes back right, the budget is never passed."""
    import torch
    from libmarshal_gb300 import lm
    specs = make_jobs(12, 60, 64, 1500)
    srcs, ins, outs = [], [], []
    for k, (op, d, e) in enumerate(specs):
        src = O.random_bits(nelems(op, d), e, 900 + k)
        srcs.append(src)
        ins.append(torch.from_numpy(src.view(np.uint8).copy()).pin_memory())
        outs.append(torch.empty_like(ins[-1]).pin_memory())
    largest = max(t.numel() for t in ins)
    budget = 2 * largest + 4096
    assert budget < sum(t.numel() for t in ins)
    srv = lm.Server(budget)
    for (op, d, e), i, o in zip(specs, ins, outs):
        srv.submit(op, d, e, src=i, dst=o)
    srv.drain(120000)
    st = srv.stats()
    res = srv.poll(10000)
    srv.close()
    assert len(res) == len(specs) and all(r[1] == 0 for r in res)
    assert st["peak_inflight_bytes"] <= budget
    assert max(r[3] for r in res) > 0  # some request waited for admission
    _check(specs, srcs, [o.numpy() for o in outs])


def test_serve_concurrent_submitters(cuda):
    """Two client threads submitting with gaps (arrivals while batches run)."""
    import torch
    from libmarshal_gb300 import lm
    specs = make_jobs(13, 120, 16, 700)
    srcs, bufs = _device_reqs(cuda, specs, 1300)
    torch.cuda.synchronize()
    srv = lm.Server(1 << 30)
    errs = []

    def client(part):
        try:
            for k in part:
                op, d, e = specs[k]
                srv.submit(op, d, e, buf=bufs[k])
                time.sleep(0.0002)
        except Exception as ex:  # reported below
            errs.append(ex)

    th = [threading.Thread(target=client, args=(range(i, len(specs), 2),))
          for i in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    srv.drain(60000)
    st = srv.stats()
    srv.close()
    assert not errs
    assert st["completed"] == len(specs)
    _check(specs, srcs, [b.cpu().numpy() for b in bufs])


def test_serve_rejects_bad_requests(cuda):
    import torch
    from libmarshal_gb300 import lm
    b = torch.zeros(1 << 20, dtype=torch.uint8, device=cuda)
    srv = lm.Server(1 << 16)
    with pytest.raises(lm.LMError):  # larger than the budget
        srv.submit(lm.OP_TRANSPOSE, (1024, 1024), 1, buf=b)
    with pytest.raises(lm.LMError):
        srv.submit(lm.OP_TRANSPOSE, (8, 8), 3, buf=b)
    srv.submit(lm.OP_TRANSPOSE, (64, 64), 1, buf=b)
    srv.drain(10000)
    srv.close()


def test_serve_poisson_trace_every_request(cuda):
    """The served configuration's trace generator (Poisson arrivals at 100k
    requests/s, seed 2, the five layout conversions, widths 1/2/4/8) with
    400 requests of 4 KiB to 64 MiB, each on its own device region with a
    seeded input: replayed at its arrival times through the server (in the
    mix, continuously batched) and one request per call (alone); every
    request's result against the oracle in both forms."""
    import torch
    import bench
    from libmarshal_gb300 import lm
    from oracle import check as C
    trace = bench.serve_trace(400, 100000.0, hi=64 << 20)
    code = {"aos_asta": C.OP_AOS_ASTA, "asta_aos": C.OP_ASTA_AOS,
            "soa_asta": C.OP_SOA_ASTA, "asta_soa": C.OP_ASTA_SOA,
            "transpose": C.OP_TRANSPOSE}
    offs, tot = [], 0
    for (_, op, d, e) in trace:
        offs.append(tot)
        tot += (C.n_elems(code[op], d) * e + 255) // 256 * 256
    arena = torch.empty(tot, dtype=torch.uint8, device=cuda)
    vjobs = [(off, code[op], d, e) for off, (_, op, d, e) in zip(offs, trace)]
    reqs, arrival = [], []
    for (t_ns, op, d, e), off in zip(trace, offs):
        r = lm.Request()
        r.elem_bytes, r.op = e, code[op]
        r.d0, r.d1, r.d2, r.d3 = list(d) + [0] * (4 - len(d))
        r.buf = arena.data_ptr() + off
        reqs.append(r)
        arrival.append(t_ns)
    for mode in ("served", "plain"):
        host = np.empty(tot, dtype=np.uint8)
        C.fill_host(host, vjobs, 8 << 20)
        arena.copy_(torch.from_numpy(host))
        del host
        torch.cuda.synchronize()
        srv = lm.Server(16 << 30) if mode == "served" else None
        res = lm.serve_replay(srv, reqs, arrival, None,
                              plain=(mode == "plain"))
        if srv is not None:
            srv.close()
        torch.cuda.synchronize()
        assert not any(r[0] for r in res), mode
        bad = C.check_host(arena.cpu().numpy(), vjobs, 8 << 20)
        assert not bad, (mode, bad[:10])
    assert lm.lib().lm_device_status(None) == 0
