"""The parse server (continuous batching): every request's result equals the
same document parsed alone and the oracle's; verdicts per request; memory
budget admission; Poisson replay."""
import numpy as np
import pytest
from tests import synth

pytestmark = pytest.mark.gpu


def alone(ctx, doc, lines):
    if lines:
        return ctx.try_parse(doc, lines=True, chunk_sizes=[doc.size])
    return ctx.try_parse(doc)


def test_results_same_alone_and_in_the_mix(cj, oracle, ctx):
    docs, lines, kinds = synth.serve_requests(0x5E4E0001, 240, median=16 << 10, max_size=4 << 20,
                                           adversarial_frac=0.02, backslash_bytes=1 << 20)
    bad = synth.synth_document(77, 30000)
    assert synth.synth_corrupt(bad, synth.CORRUPT_OVERLONG3, 1)
    docs.insert(17, bad)
    lines = np.insert(lines, 17, False)
    with cj.Server(slots=2, max_batch_docs=64, memory_budget=2 << 30) as srv:
        tickets = [srv.submit(d, bool(l)) for d, l in zip(docs, lines)]
        results = [srv.take(t) for t in tickets]
        stats = srv.stats().as_dict()
    assert stats["batches"] >= 4 and stats["fault"] == 0
    for i, (d, l) in enumerate(zip(docs, lines)):
        st, res = results[i]
        st1, res1 = alone(ctx, d, bool(l))
        assert st == st1, i
        ref = oracle.parse(d, lines=bool(l), chunk_sizes=[d.size] if l else None)
        if st == cj.OK:
            np.testing.assert_array_equal(res.buffer, res1.buffer, err_msg=f"request {i}")
            np.testing.assert_array_equal(res.buffer, ref.reference_layout(), err_msg=f"request {i}")
        else:
            assert ref.flags != 0
    assert results[17][0] == cj.ERR_INVALID_UTF8


def test_replay_poisson(cj):
    docs, lines, _ = synth.serve_requests(0x5E4E0002, 300, median=8 << 10, max_size=1 << 20,
                                       adversarial_frac=0.0)
    rng = np.random.default_rng(3)
    arrivals = np.cumsum(rng.exponential(1 / 5000.0, len(docs)))
    with cj.Server(slots=2, max_batch_docs=256) as srv:
        status, lat, makespan = srv.replay(docs, lines, arrivals)
        stats = srv.stats()
    assert (status == cj.OK).all()
    assert (lat > 0).all() and makespan >= arrivals[-1]
    assert stats.docs == len(docs) and stats.batches >= 2


def test_memory_budget_admission(cj):
    budget = 64 << 20                     # 32 MiB of device bytes per slot
    docs, lines, _ = synth.serve_requests(0x5E4E0003, 120, median=64 << 10, max_size=512 << 10,
                                       adversarial_frac=0.0)
    with cj.Server(slots=2, max_batch_docs=1024, memory_budget=budget) as srv:
        tickets = [srv.submit(d, bool(l)) for d, l in zip(docs, lines)]
        for t in tickets:
            assert srv.take(t)[0] == cj.OK
        st = srv.stats()
        assert st.peak_admitted_bytes <= budget // 2
        assert st.batches > 2
        big = synth.synth_document(5, 4 << 20)
        with pytest.raises(cj.CujsonError):
            srv.submit(big)               # more than a slot's share of the budget
