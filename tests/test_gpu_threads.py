"""Engines are independent: host threads that each drive their own engine
(own stream, own scratch) concurrently get exactly the results of serial
runs, and the reference-signature calls, which share one internal engine
behind a lock, can be called from several threads at once."""
import threading

import numpy as np
import pytest

from conftest import cfgs, pkg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_engines_on_concurrent_host_threads():
    P = pkg()
    jobs = [(cfgs().workload(2, 20000), 1), (cfgs().workload(4, 30000), 2),
            (cfgs().workload(3, 2000), 3), (cfgs().workload(5, 256), 4)]
    inputs = [O.normals_f32(seed, c.paths, c.nmat) for c, seed in jobs]

    def run(c, z):
        with P.Engine(c) as e:
            g, _ = e.greeks_f32(z)
        return g

    serial = [run(c, z) for (c, _), z in zip(jobs, inputs)]
    results = [None] * len(jobs)
    errors = []

    def worker(k):
        try:
            for _ in range(3):
                results[k] = run(jobs[k][0], inputs[k])
        except Exception as ex:     # reported below
            errors.append(ex)

    threads = [threading.Thread(target=worker, args=(k,)) for k in range(len(jobs))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for a, b in zip(results, serial):
        np.testing.assert_array_equal(a, b)


def test_reference_signature_from_several_threads():
    P = pkg()
    ref = P.swaption_greeks(4096)
    out, errors = [], []

    def worker():
        try:
            out.append(P.swaption_greeks(4096))
        except Exception as ex:
            errors.append(ex)

    threads = [threading.Thread(target=worker) for _ in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for z, v, lb in out:
        np.testing.assert_array_equal(z, ref[0])
        assert v == ref[1] and lb == ref[2]
