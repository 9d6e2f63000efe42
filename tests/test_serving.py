"""Serving form (rsg_server_*): continuous batching of independent systems. Each result must be the same alone
and in the mix (every request has its own plan and the kernels are deterministic: bit for bit), and admission
must respect the device-memory budget."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def requests(k, seed, lo=1e3, hi=3e4):
    from ressim_gb300 import synth
    rng = np.random.default_rng(seed)
    return [synth.serving_request(rng, cells_lo=lo, cells_hi=hi) for _ in range(k)]


def true_res(A, x, b):
    from ressim_gb300 import synth
    return np.linalg.norm(b - synth.bsr_matvec_host(A, x)) / np.linalg.norm(b)


@pytest.mark.parametrize("precond,precision", [("cpr", "mixed_f32"), ("bilu0", "fp64")])
def test_result_is_the_same_alone_and_in_the_mix(precond, precision):
    from ressim_gb300.solver import Server
    reqs = requests(6, seed=11)
    alone = []
    with Server(slots=1, precond=precond, precision=precision) as s:
        for r in reqs:
            alone.append(s.poll(s.submit(r.A, r.b, tol=1e-6, maxit=500)))
    with Server(slots=4, precond=precond, precision=precision) as s:
        ids = [s.submit(r.A, r.b, tol=1e-6, maxit=500) for r in reqs]       # all arrive while others run
        mix = [s.poll(i) for i in ids]
    slots, conv, shared = set(), 0, 0
    for r, (xa, ra), (xm, rm) in zip(reqs, alone, mix):
        # same status, iterations and iterate bit for bit (also for a request that does not converge: the generator
        # draws some that FP64 CPR / BILU0 with BiCGSTAB or GMRES cannot solve either, e.g. the second one here)
        assert ra["status"] == rm["status"] and ra["iterations"] == rm["iterations"]
        assert np.array_equal(xa, xm, equal_nan=True)
        if rm["status"] == 0:
            assert true_res(r.A, xm, r.b) <= 1e-5
            conv += 1
        slots.add(rm["slot"])
        shared += rm["batch"] > 1
    assert conv >= 5
    assert len(slots) > 1 or shared > 1                                 # the mix really shared the device


def test_small_requests_are_batched():
    """Small requests queued together are solved in one block-diagonal launch; each result is bit for bit the one it
    has alone, and the batch really formed."""
    from ressim_gb300.solver import Server
    reqs = requests(8, seed=21, lo=1e3, hi=1.5e4)
    with Server(slots=1, precond="cpr", precision="mixed_f32") as s:
        alone = [s.poll(s.submit(r.A, r.b, tol=1e-6, maxit=500)) for r in reqs]
    with Server(slots=1, precond="cpr", precision="mixed_f32") as s:
        ids = [s.submit(r.A, r.b, tol=1e-6, maxit=500) for r in reqs]
        mix = [s.poll(i) for i in ids]
    assert max(rm["batch"] for _, rm in mix) > 1
    for (xa, ra), (xm, rm) in zip(alone, mix):
        assert ra["batch"] == 1
        assert ra["status"] == rm["status"] and ra["iterations"] == rm["iterations"]
        assert np.array_equal(xa, xm, equal_nan=True)


def test_admission_respects_the_budget():
    from ressim_gb300 import synth
    from ressim_gb300.solver import Server
    reqs = [synth.make_system(24, 24, 6, sigma=1.0, seed=s, wells="corners+center") for s in range(4)]
    with Server(slots=4) as probe:
        need = max(probe.request_bytes(r.A) for r in reqs)
    with Server(slots=4, mem_budget=int(1.5 * need)) as s:                  # one request at a time fits
        ids = [s.submit(r.A, r.b, tol=1e-6, maxit=300) for r in reqs]
        res = [s.poll(i)[1] for i in ids]
    spans = sorted((r["start_ms"], r["end_ms"]) for r in res)           # the server's clock
    for (a0, a1), (b0, b1) in zip(spans, spans[1:]):
        assert b0 >= a1                                                 # admitted only after the previous one left
    assert all(r["status"] == 0 for r in res)


def test_oversized_request_is_rejected():
    from ressim_gb300 import _lib, synth
    from ressim_gb300.solver import Server
    A = synth.make_system(16, 16, 4, seed=1).A
    with Server(slots=1, mem_budget=1 << 20) as s:
        with pytest.raises(_lib.RsgError) as e:
            s.submit(A, np.ones(A.n * 3))
        assert e.value.code == _lib.RSG_ENOMEM


def test_poll_without_wait_and_load():
    from ressim_gb300.solver import Server
    reqs = requests(3, seed=5)
    with Server(slots=2) as s:
        ids = [s.submit(r.A, r.b) for r in reqs]
        q, running, inuse = s.load()
        assert q + running <= 3 and inuse >= 0
        import time
        done = {}
        for _ in range(60000):                                          # at most about a minute
            time.sleep(0.001)
            for i in ids:
                if i not in done:
                    out = s.poll(i, wait=False)
                    if out is not None:
                        done[i] = out
            if len(done) == len(ids):
                break
        assert len(done) == len(ids)
        q, running, resident = s.load()
        assert (q, running) == (0, 0)
        assert resident >= 0                     # the idle slots' resident plans (released when an admission needs room)


def test_held_requests_are_admitted_together():
    """Requests submitted while admission is held (rsg_server_hold) wait in the queue and are then solved as one batch,
    each with the result it has alone."""
    from ressim_gb300.solver import Server
    reqs = requests(5, seed=31, lo=1e3, hi=1.2e4)
    with Server(slots=1, precond="cpr", precision="mixed_f32") as s:
        alone = [s.poll(s.submit(r.A, r.b, tol=1e-6, maxit=500)) for r in reqs]
    with Server(slots=1, precond="cpr", precision="mixed_f32") as s:
        s.hold(True)
        ids = [s.submit(r.A, r.b, tol=1e-6, maxit=500) for r in reqs]
        q, running, _ = s.load()
        assert running == 0 and q == len(reqs)                          # nothing admitted while held
        s.hold(False)
        mix = [s.poll(i) for i in ids]
    assert max(rm["batch"] for _, rm in mix) == len(reqs)
    for (xa, ra), (xm, rm) in zip(alone, mix):
        assert ra["status"] == rm["status"] and ra["iterations"] == rm["iterations"]
        assert np.array_equal(xa, xm, equal_nan=True)


def test_lent_arrays_give_the_copied_result():
    """rsg_submit_view reads the caller's arrays in place instead of copying them: every result (alone and in a held
    batch) is bit for bit the one rsg_submit gives, and the Python mirror keeps the lent arrays until they are
    polled."""
    from ressim_gb300.solver import Server
    reqs = requests(4, seed=41, lo=1e3, hi=1.2e4)
    with Server(slots=1, precond="cpr", precision="mixed_f32") as s:
        s.hold(True)
        ids = [s.submit(r.A, r.b, tol=1e-6, maxit=500) for r in reqs]
        s.hold(False)
        copied = [s.poll(i) for i in ids]
        lent_alone = [s.poll(s.submit(r.A, r.b, tol=1e-6, maxit=500, copy=False)) for r in reqs]
        s.hold(True)
        ids = [s.submit(r.A, r.b, tol=1e-6, maxit=500, copy=False) for r in reqs]
        assert len(s.lent) == len(reqs)
        s.hold(False)
        lent_batch = [s.poll(i) for i in ids]
        assert not s.lent
    assert max(rm["batch"] for _, rm in copied) == len(reqs)
    assert max(rm["batch"] for _, rm in lent_batch) == len(reqs)
    for (xc, rc), (xa, ra), (xb, rb) in zip(copied, lent_alone, lent_batch):
        assert rc["status"] == ra["status"] == rb["status"]
        assert rc["iterations"] == ra["iterations"] == rb["iterations"]
        assert np.array_equal(xc, xa, equal_nan=True) and np.array_equal(xc, xb, equal_nan=True)
