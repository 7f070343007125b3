"""Serving form: several sessions behind one request queue on one GPU
(include/gpumap_gb300_server.h, gpumap_gb300/serving.py).

* A session's k-NN lists are the same whether its requests run alone or
  interleaved with other sessions' requests on several slots; its embedding
  agrees in trustworthiness within 0.015 (the SGD's concurrent updates land
  in a different order).
* Admission: a session beyond the device-memory budget, rows beyond a
  session's capacity and unknown ids are refused with the stated codes.
"""
import numpy as np
import pytest

from gpumap_gb300.datasets import mixture_stream
from oracle.knn import exact_knn, recall_at_k, trustworthiness

pytestmark = pytest.mark.gpu

F32, I32 = np.float32, np.int32


def _params(native, n, d, k=10, precision=1, overlap=1, max_epoch=200):
    p = native.default_params(n_instances=n, n_features=d, n_neighbors=k, max_epoch=max_epoch,
                              precision=precision, overlap=overlap)
    p.a, p.b = 1.5769434602697652, 0.8950608778515733
    return p


SPECS = [(3000, 32, 5, 0), (5000, 64, 8, 1), (4000, 24, 6, 2)]  # n, d, centres, seed


def _data():
    return [np.concatenate(list(mixture_stream(n, d, c, s))) for n, d, c, s in SPECS]


def _requests(data, size=500, seed=0):
    # every session's rows cut into requests of `size`, interleaved at random
    rng = np.random.default_rng(seed)
    order = np.concatenate([np.full(len(x) // size, i) for i, x in enumerate(data)])
    rng.shuffle(order)
    cursor = [0] * len(data)
    out = []
    for i in order:
        out.append((int(i), data[i][cursor[i]: cursor[i] + size]))
        cursor[i] += size
    return out


def _tables(sess, n, k):
    return sess.copy("knn_ids", I32)[: n * k].reshape(n, k), sess.copy("pub_idx", np.uint32).reshape(-1, k + 1)[:n, :k]


@pytest.mark.parametrize("precision", [1, 0])
def test_session_results_alone_equal_mix(native, precision):
    from gpumap_gb300.serving import Server

    data = _data()
    reqs = _requests(data)
    k = 10
    # in the mix: three slots, requests of all sessions interleaved
    with Server(slots=3, hbm_budget=50 * 10**9) as srv:
        sids = [srv.open_session(_params(native, len(x), x.shape[1], k, precision)) for x in data]
        rids = [srv.submit(sids[i], rows, len(rows), len(rows)) for i, rows in reqs]
        # a last cycle per session embeds every row (its lists are final)
        rids += [srv.submit(sids[i], np.zeros((0, x.shape[1]), F32), 0, len(x)) for i, x in enumerate(data)]
        infos = [srv.wait(r) for r in rids]
        assert all(inf.status == 0 for inf in infos)
        mix = []
        for i, x in enumerate(data):
            s = srv.session(sids[i])
            mix.append((*_tables(s, len(x), k), s.copy("embedding", F32).reshape(-1, 2)[: len(x)]))
        st = srv.stats()
        assert st.finished == len(reqs) + len(data) and st.failed == 0
        assert st.rows == sum(len(x) for x in data)
        assert st.latency_p99 >= st.latency_p50 > 0
    # alone: each session's requests in the same order, one slot, nothing else queued
    for i, x in enumerate(data):
        with Server(slots=1, hbm_budget=50 * 10**9) as srv:
            sid = srv.open_session(_params(native, len(x), x.shape[1], k, precision))
            for j, rows in reqs:
                if j == i:
                    assert srv.wait(srv.submit(sid, rows, len(rows), len(rows))).status == 0
            assert srv.wait(srv.submit(sid, np.zeros((0, x.shape[1]), F32), 0, len(x))).status == 0
            s = srv.session(sid)
            ids, pub = _tables(s, len(x), k)
            emb = s.copy("embedding", F32).reshape(-1, 2)[: len(x)]
        np.testing.assert_array_equal(mix[i][0], ids)
        np.testing.assert_array_equal(mix[i][1], pub)
        # the embedding after the full last cycle (each cycle before it embeds
        # only its new rows and smooths the rest): same lists, SGD updates in
        # a different order; the stated tolerance is 0.015
        sample = np.arange(0, len(x), 4)
        t_mix = trustworthiness(x, mix[i][2], k, sample=sample)
        t_alone = trustworthiness(x, emb, k, sample=sample)
        assert abs(t_mix - t_alone) <= 0.015, (i, t_mix, t_alone)
        if precision == 1:
            q = np.arange(0, len(x), 7)
            ei, _ = exact_knn(x, k, queries=q)
            assert recall_at_k(pub[q], ei) >= 0.99


def test_server_admission_and_errors(native):
    from gpumap_gb300.serving import Server

    with Server(slots=2, hbm_budget=512 * 2**20) as srv:  # 512 MiB
        with pytest.raises(native.GMError) as e:
            srv.open_session(_params(native, 200_000, 128))
        assert e.value.code == native.GM_ERR_CAPACITY
        sid = srv.open_session(_params(native, 1000, 8, k=5))
        x = np.random.default_rng(0).normal(size=(1200, 8)).astype(F32)
        assert srv.wait(srv.submit(sid, x[:600], 600, 600)).status == 0
        with pytest.raises(native.GMError) as e:  # 600 + 600 > n_instances
            srv.submit(sid, x[600:1200], 0, 0)
        assert e.value.code == native.GM_ERR_CAPACITY
        with pytest.raises(ValueError):  # wrong width
            srv.submit(sid, x[:10, :4], 0, 0)
        with pytest.raises(ValueError):
            srv.wait(987654)
        with pytest.raises(ValueError):
            srv.submit(424242, x[:10], 0, 0)
        assert srv.wait(srv.submit(sid, x[600:1000], 400, 400)).status == 0
        srv.close_session(sid)
        assert srv.stats().sessions_open == 0 and srv.stats().bytes_in_use == 0
