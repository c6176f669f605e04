"""The serving form (ftx_server_*): each request's result is the same run
alone and in a concurrent mix (bit-exact; integer arithmetic, so the
tolerance is zero), matches the plain drop-in calls, and admission honours
the HBM budget."""
import numpy as np
import pytest

from libftcrypto_gb300 import synth

pytestmark = pytest.mark.gpu


def make_requests(ft, g, pk, nreq=16):
    reqs = []
    for i in range(nreq):
        op = ("encrypt", "rerand", "smul", "segsum")[i % 4]
        n = int(g.integers(50, 3000))
        r = synth.scalars_mod_L(g, n)
        if op == "encrypt":
            reqs.append({"op": op, "m": synth.plaintexts(g, n, 1), "r": r})
            continue
        base1, base2 = ft.encrypt(pk, synth.plaintexts(g, n, 1), r, 1)
        req = {"op": op, "c": (base1, base2)}
        if op == "rerand":
            req["r"] = synth.scalars_mod_L(g, n)
        elif op == "smul":
            req["k"] = synth.scalars_mod_L(g, n)
        else:
            req["off"] = synth.csr_offsets(g, n, max(1, n // 32))
        reqs.append(req)
    return reqs


def submit(srv, req):
    if req["op"] == "encrypt":
        return srv.submit_encrypt(req["m"], req["r"], 1)
    c1, c2 = (x.get_range(0, len(x), 1) for x in req["c"])  # fresh copies for in-place ops
    if req["op"] == "rerand":
        return srv.submit_rerand(c1, c2, req["r"])
    if req["op"] == "smul":
        return srv.submit_smul(c1, c2, req["k"])
    return srv.submit_segsum(c1, c2, req["off"])


def folded(pair):
    return np.concatenate([pair[0].to_bytes_folded(), pair[1].to_bytes_folded()])


def test_alone_equals_mix_equals_plain(ft, orc):
    g = synth.rng(41)
    sk = synth.scalars_mod_L(g, 1)
    pk = orc.encode(orc.from_scalars(sk))[0]
    reqs = make_requests(ft, g, pk)
    srv = ft.Server(pk, 8 << 30, slots=6)
    alone = []
    for req in reqs:
        c1, c2, _, _ = srv.wait(submit(srv, req))
        alone.append(folded((c1, c2)))
    tickets = [submit(srv, req) for req in reqs]  # all in flight together
    mixed = [folded(srv.wait(t)[:2]) for t in tickets]
    for a, b in zip(alone, mixed):
        assert (a == b).all()
    # the plain drop-in calls give the same ciphertexts
    for req, a in zip(reqs, alone):
        if req["op"] == "encrypt":
            p = ft.encrypt(pk, req["m"], req["r"], 1)
        else:
            p = tuple(x.get_range(0, len(x), 1) for x in req["c"])
            if req["op"] == "rerand":
                z = ft.encrypt(pk, np.zeros(len(p[0]), np.uint64), req["r"], 1)
                p[0].add(z[0])
                p[1].add(z[1])
            elif req["op"] == "smul":
                p[0].mul(req["k"])
                p[1].mul(req["k"])
            else:
                p = (ft.segmented_sum_csr(req["off"], p[0]), ft.segmented_sum_csr(req["off"], p[1]))
        assert (folded(p) == a).all(), req["op"]
    srv.close()


def test_budget_admission(ft, orc):
    g = synth.rng(42)
    pk = orc.encode(orc.from_scalars(synth.scalars_mod_L(g, 1)))[0]
    n = 20000
    per_req = 2 * n * 128 + n * 40 + 4096  # device bytes of one encrypt request
    srv = ft.Server(pk, per_req + 1000, slots=4)  # room for one request at a time
    m = synth.plaintexts(g, n, 1)
    r = synth.scalars_mod_L(g, n)
    ts = [srv.submit_encrypt(m, r, 1) for _ in range(4)]
    used, queued, running = srv.stats()
    assert running <= 1 and used <= per_req + 1000
    outs = []
    for t in ts:  # each output handed back before the next request can fit
        c1, c2 = srv.wait(t)[:2]
        outs.append(folded((c1, c2)))
        srv.release(c1, c2)
    assert all((o == outs[0]).all() for o in outs)
    assert srv.stats()[0] == 0
    with pytest.raises(ft.FtError) as e:
        srv.submit_encrypt(np.zeros(2 * n, np.uint64), synth.scalars_mod_L(g, 2 * n), 1)
    assert e.value.code == 7  # larger than the whole budget
    srv.close()


def test_submit_checks_and_close_with_results_pending(ft, orc):
    g = synth.rng(43)
    pk = orc.encode(orc.from_scalars(synth.scalars_mod_L(g, 1)))[0]
    srv = ft.Server(pk, 1 << 30, slots=2)
    r = synth.scalars_mod_L(g, 4)
    with pytest.raises(ft.FtError) as e:  # a plaintext above its stated bound
        srv.submit_encrypt(np.array([0, 1, 2, 1], np.uint64), r, 1)
    assert e.value.code == 3
    t = srv.submit_encrypt(np.array([0, 1, 1, 0], np.uint64), r, 1)
    want = folded(ft.encrypt(pk, np.array([0, 1, 1, 0], np.uint64), r, 1))
    assert (folded(srv.wait(t)[:2]) == want).all()
    for _ in range(3):  # never collected: freed with the server
        srv.submit_encrypt(synth.plaintexts(g, 1000, 1), synth.scalars_mod_L(g, 1000), 1)
    srv.close()


def test_budget_counts_resident_outputs(ft, orc):
    """Outputs the server created hold their bytes of the budget until they
    are released: with room for two outputs, a third encrypt waits while the
    first two are kept, and is admitted once one of them is released."""
    import time
    g = synth.rng(44)
    pk = orc.encode(orc.from_scalars(synth.scalars_mod_L(g, 1)))[0]
    n = 10000
    out_bytes = 2 * n * 128                # the two arrays an encrypt creates
    tmp_bytes = n * 40 + 4096              # its staged inputs while it runs
    srv = ft.Server(pk, 2 * out_bytes + tmp_bytes + 1000, slots=4)
    m = synth.plaintexts(g, n, 1)
    r = synth.scalars_mod_L(g, n)
    want = folded(ft.encrypt(pk, m, r, 1))
    t1, t2 = srv.submit_encrypt(m, r, 1), srv.submit_encrypt(m, r, 1)
    a1, a2 = srv.wait(t1)[:2], srv.wait(t2)[:2]
    assert srv.stats()[0] == 2 * out_bytes
    t3 = srv.submit_encrypt(m, r, 1)
    deadline = time.time() + 1.0
    while time.time() < deadline:          # the third stays queued: no room
        used, queued, running = srv.stats()
        assert (queued, running) == (1, 0) and used == 2 * out_bytes
        time.sleep(0.05)
    srv.release(*a1)                       # room for one more output
    a3 = srv.wait(t3)[:2]
    for a in (a2, a3):
        assert (folded(a) == want).all()
    srv.release(*a2)
    srv.release(*a3)
    assert srv.stats() == (0, 0, 0)
    # arrays the server does not hold are refused
    other = ft.Array.init_scalar(3)
    assert ft.api.lib().ftx_server_release(srv._h, other.handle) == 4  # FT_ERR_OUT_OF_BOUNDS
    srv.close()
