"""Interruption and concurrent callers (GPU).

The reference checks its context at every Newton iteration, time step and
frequency and returns "analysis interrupted" wrapping ctx.Err()
(analysis/op.go:81-89).  The engine has the two forms a Go wrapper needs: a
per-call wall-clock deadline measured on the device (ks_options.deadline_s) and
a cancel word the host writes while kernels run (ks_batch_cancel_word).  Both
end unfinished circuits with KS_STATUS_INTERRUPTED through bounded checks in
the kernels' own loops: nothing spins.  Separate batches may be driven from
separate host threads at once (one handle per goroutine).
"""
import threading
import time

import numpy as np
import pytest

from kronspice_gb300 import analysis, build, workloads

pytestmark = pytest.mark.gpu
INTERRUPTED = 6


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


@pytest.fixture(scope="module")
def opamps():
    el, nn, vals = workloads.cmos_opamp_batch(65536, seed=0)
    return analysis.Batch(analysis.Plan(el, nn, vals.shape[1]), vals)


def test_deadline_interrupts_unfinished_circuits(opamps):
    """A 1 us deadline on 65,536 op-amps (a ~0.5 s solve from InitJct): the call
    returns at once and the circuits it did not finish report the typed
    interruption; with no deadline every circuit converges."""
    t0 = time.perf_counter()
    x, st, it = opamps.op(analysis.Options(reltol=1e-6, deadline_s=1e-6, kernel="generic"))
    wall = time.perf_counter() - t0
    assert set(np.unique(st)) <= {0, INTERRUPTED}
    assert (st == INTERRUPTED).mean() > 0.9
    assert wall < 0.25, wall
    assert isinstance(analysis.status_error(INTERRUPTED), analysis.ErrInterrupted)
    x, st, it = opamps.op(analysis.Options(reltol=1e-6, kernel="generic"))
    assert np.all(st == 0)


def test_cancel_word_interrupts_a_running_solve(opamps):
    word = opamps.cancel_word()
    opt = analysis.Options(reltol=1e-6, kernel="generic")
    # set before the call: nothing runs to completion
    word.value = 1
    x, st, it = opamps.op(opt)
    assert np.all(st == INTERRUPTED)
    word.value = 0
    t0 = time.perf_counter()
    x, st, it = opamps.op(opt)
    full = time.perf_counter() - t0
    assert np.all(st == 0)
    # set while the kernel runs, from another thread: the solve ends early and
    # the circuits it had not finished are interrupted
    timer = threading.Timer(0.2 * full, lambda: setattr(word, "value", 1))
    t0 = time.perf_counter()
    timer.start()
    x, st, it = opamps.op(opt)
    cut = time.perf_counter() - t0
    timer.join()
    word.value = 0
    assert set(np.unique(st)) <= {0, INTERRUPTED}
    assert (st == INTERRUPTED).any() and (st == 0).any()
    assert cut < 0.8 * full, (cut, full)
    x, st, it = opamps.op(opt)
    assert np.all(st == 0)


def test_batches_from_four_host_threads():
    """Four host threads, one batch each, solving at the same time: the same
    results as one after another."""
    batches = []
    for k in range(4):
        el, nn, vals = workloads.bjt_ce_batch(4096, seed=40 + k)
        batches.append(analysis.Batch(analysis.Plan(el, nn, vals.shape[1]), vals))
    opt = analysis.Options(reltol=1e-6, precision="mixed", kernel="generic")
    seq = [b.op(opt) for b in batches]
    out = [None] * 4
    errs = []

    def run(k):
        try:
            for _ in range(3):
                out[k] = batches[k].op(opt)
        except Exception as e:  # noqa: BLE001 - reported below
            errs.append(e)
    threads = [threading.Thread(target=run, args=(k,)) for k in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errs, errs
    for k in range(4):
        for a, b in zip(seq[k], out[k]):
            assert np.array_equal(a, b)
