"""GPU: the serving loop (iwpp_server_*).  Every request's result must be the
same bytes alone (one request in flight) and in a mix of concurrent requests
of different sizes, pixel types and connectivities, and equal the CPU oracle;
admission must keep the device bytes of admitted requests within the budget."""
import threading

import numpy as np
import pytest

import iwpp
import oracle
from iwpp import synth

pytestmark = pytest.mark.gpu


def _requests():
    """A mix of small and medium requests: uint8 / uint16 / int32, 4- and
    8-connectivity, h-dome and sparse-seed markers, ragged shapes."""
    rng = np.random.default_rng(44)
    shapes = [(1, 1), (7, 300), (256, 256), (300, 7), (513, 257), (640, 480), (1000, 333), (129, 1500),
              (1024, 1024), (2, 4096), (777, 901), (64, 128)]
    reqs = []
    for i, (h, w) in enumerate(shapes):
        dt = [0, 0, 1, 2][i % 4]
        conn = 8 if i % 3 else 4
        mask = synth.noise_mask(w, h, dt, 400 + i, 3.0, 4)
        if i % 2:
            marker = synth.sparse_marker(mask, 500 + i, 0.001)
        else:
            marker = synth.hdome_marker(mask, int(rng.integers(5, 121)))
        reqs.append((marker, mask, conn))
    return reqs


@pytest.fixture(scope="module")
def reqs_and_refs():
    reqs = _requests()
    refs = [oracle.reconstruct(m, k, c) for m, k, c in reqs]
    return reqs, refs


def test_each_result_same_alone_and_in_the_mix(reqs_and_refs):
    reqs, refs = reqs_and_refs
    with iwpp.Server(lanes=3) as srv:
        alone = []
        for m, k, c in reqs:
            out, info = srv.wait(srv.submit(m, k, c))
            assert info["status"] == 0 and info["batch_size"] == 1
            alone.append(out)
        # the mix: everything submitted at once, three times over
        tickets = [srv.submit(m, k, c) for _ in range(3) for m, k, c in reqs]
        mixed = [srv.wait(t) for t in tickets]
        st = srv.stats()
    for i, ref in enumerate(refs):
        assert np.array_equal(alone[i], ref), i
        for rep in range(3):
            out, info = mixed[rep * len(reqs) + i]
            assert info["status"] == 0
            assert np.array_equal(out, ref), (rep, i)
    assert st["completed"] == 4 * len(reqs) and st["failed"] == 0
    assert st["largest_batch"] > 1  # the mix did batch
    assert st["bytes_in_use"] == 0


def test_submissions_from_many_threads(reqs_and_refs):
    reqs, refs = reqs_and_refs
    results = {}
    with iwpp.Server(lanes=2, max_batch=5) as srv:
        def client(j):
            for i in range(j, len(reqs), 4):
                m, k, c = reqs[i]
                results[i] = srv.wait(srv.submit(m, k, c))[0]
        ths = [threading.Thread(target=client, args=(j,)) for j in range(4)]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
    for i, ref in enumerate(refs):
        assert np.array_equal(results[i], ref), i


def test_admission_stays_within_the_memory_budget(reqs_and_refs):
    reqs, refs = reqs_and_refs
    # room for the largest request and little more: requests queue for memory
    budget = 3 * 1024 * 1024 * 4
    with iwpp.Server(lanes=3, memory_budget=budget) as srv:
        tickets = [srv.submit(m, k, c) for m, k, c in reqs for _ in range(2)]
        outs = [srv.wait(t)[0] for t in tickets]
        st = srv.stats()
    assert st["bytes_peak"] <= budget
    assert st["memory_budget"] == budget
    for i, out in enumerate(outs):
        assert np.array_equal(out, refs[i // 2]), i


def test_admission_sees_device_memory_taken_after_creation():
    # Admission checks the device's free memory when a request comes up, not
    # only the budget fixed at creation: memory another user of the device
    # takes after the server started holds requests back until it is given
    # back.
    import torch
    mask = synth.noise_mask(4096, 4096, 1, 31, 2.0, 3)   # uint16: a 64 MiB request
    marker = synth.sparse_marker(mask, 32, 1e-4)
    ref = oracle.reconstruct(marker, mask, 8)
    mib = 1 << 20
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    free0, _ = torch.cuda.mem_get_info()
    # after creation the server's pool holds its 256 MiB budget unused, so the
    # room it sees is the free memory before creation less this headroom:
    # about 1 GiB
    with iwpp.Server(lanes=1, memory_budget=256 * mib, memory_headroom=free0 - 1024 * mib) as srv:
        out, info = srv.wait(srv.submit(marker, mask, 8))
        assert info["status"] == 0 and np.array_equal(out, ref)
        held0 = srv.stats()["held_back"]
        # another tenant takes all but ~30 MiB of that room
        block = torch.empty(1024 * mib - 32 * mib, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        t = srv.submit(marker, mask, 8)
        with pytest.raises(TimeoutError):  # not finished: held back
            srv.wait(t, timeout_ms=300)
        assert srv.stats()["held_back"] > held0
        # ... and gives it back: the request is admitted and served
        del block
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        out, info = srv.wait(t, timeout_ms=60000)
        assert info["status"] == 0 and np.array_equal(out, ref)


def test_request_larger_than_the_budget_is_refused():
    mask = synth.noise_mask(2048, 2048, 0, 9, 2.0, 3)
    marker = synth.hdome_marker(mask, 30)
    with iwpp.Server(lanes=1, memory_budget=1 << 20) as srv:
        with pytest.raises(iwpp.IwppError) as e:
            srv.submit(marker, mask, 8)
        assert e.value.status == 8
        assert srv.stats()["rejected"] == 1


def test_pending_limit_and_strided_host_buffers():
    mask_full = synth.noise_mask(600, 400, 1, 12, 2.0, 3)
    marker_full = synth.sparse_marker(mask_full, 13, 0.002)
    # views with a row pitch larger than the row (every second column band)
    mask = mask_full[:, 100:500]
    marker = np.ascontiguousarray(marker_full)[:, 100:500]
    out = np.zeros((400, 600), np.uint16)[:, 50:450]
    ref = oracle.reconstruct(np.ascontiguousarray(marker), np.ascontiguousarray(mask), 8)
    with iwpp.Server(lanes=1, max_pending=1) as srv:
        got, info = srv.wait(srv.submit(marker, mask, 8, out=out))
        assert info["status"] == 0
        assert got is out and np.array_equal(out, ref)
        busy = 0
        tickets = []
        for _ in range(40):
            try:
                tickets.append(srv.submit(marker, mask, 8))
            except iwpp.IwppError as e:
                assert e.status == 7
                busy += 1
        for t in tickets:
            assert np.array_equal(srv.wait(t)[0], ref)
        assert srv.stats()["rejected"] == busy


def test_empty_request_completes():
    a = np.zeros((0, 5), np.uint8)
    with iwpp.Server(lanes=1) as srv:
        out, info = srv.wait(srv.submit(a, a, 8))
        assert info["status"] == 0 and out.shape == (0, 5)


def test_two_waiters_on_one_ticket():
    # one waiter gets the result, the other IWPP_ERR_INVALID; neither reads
    # a request the other has released
    mask = synth.noise_mask(2048, 2048, 0, 21, 3.0, 5)
    marker = synth.hdome_marker(mask, 60)
    ref = oracle.reconstruct(marker, mask, 8)
    lib = iwpp.load()
    with iwpp.Server(lanes=1) as srv:
        for _ in range(3):
            out = np.zeros_like(mask)
            t = srv.submit(marker, mask, 8, out=out)
            statuses = []

            def waiter():
                r = iwpp.RequestResult()
                statuses.append(lib.iwpp_server_wait(srv._p, t, -1, __import__("ctypes").byref(r)))

            ths = [threading.Thread(target=waiter) for _ in range(2)]
            for th in ths:
                th.start()
            for th in ths:
                th.join()
            assert sorted(statuses) == [0, 1]
            assert np.array_equal(out, ref)
            with pytest.raises(iwpp.IwppError):
                srv.wait(t)  # forgotten
