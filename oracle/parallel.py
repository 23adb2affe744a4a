"""The oracle's field evaluation spread over the host cores -- TEST
INFRASTRUCTURE (the timed CPU legs of bench.py).

``kriging.evaluate`` is numpy element-wise work and runs on one core; the
build's LU already uses every core through BLAS.  ``FieldPool`` splits a point
set over one worker process per core (``spawn``: safe after CUDA has started
in the parent), each worker single-threaded, and returns the field in the
original point order.  The workers start, import the oracle and receive the
series before any timed call; each call sends the points and that step's
weights.
"""
import multiprocessing as mp
import os
from concurrent.futures import ProcessPoolExecutor

import numpy as np

_SERIES = None
_THREAD_VARS = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")


def _init(series):
    global _SERIES
    _SERIES = series


def _evaluate(task):
    from . import kriging
    x, w = task
    return kriging.evaluate(_SERIES, w, x)


def host_cores():
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()


class FieldPool:
    def __init__(self, series, workers=None):
        self.workers = int(workers or host_cores())
        saved = {k: os.environ.get(k) for k in _THREAD_VARS}
        for k in _THREAD_VARS:           # children inherit this at spawn: one thread each
            os.environ[k] = "1"
        try:
            self._ex = ProcessPoolExecutor(max_workers=self.workers, mp_context=mp.get_context("spawn"),
                                           initializer=_init, initargs=(series,))
            w0 = np.zeros(series.size)
            list(self._ex.map(_evaluate, [(np.zeros((1, 3)), w0)] * self.workers))   # start every worker
        finally:
            for k, v in saved.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v

    def evaluate(self, x, w):
        """Field at x (n, 3) with weights w, over all workers."""
        parts = np.array_split(np.asarray(x, dtype=np.float64), 4 * self.workers)
        w = np.asarray(w, dtype=np.float64)
        return np.concatenate(list(self._ex.map(_evaluate, [(p, w) for p in parts if len(p)])))

    def close(self):
        self._ex.shutdown()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
