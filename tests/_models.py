"""Shared fixtures: golden-vector models and oracle adapters for the tests."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def oracle_series_from_golden(g):
    """The single series of a one-series fixture."""
    from oracle import inputs
    series, _, _ = inputs.series_from_golden(g)
    assert len(series) == 1
    return series[0]


def golden_extent(g):
    from oracle import inputs
    return inputs.golden_extent(g)


def oracle_series_list(model):
    """Oracle Series objects of a gempy_gb300 synthetic model (same split as the engine)."""
    from oracle import inputs
    return inputs.series_from_engine_inputs(model.interpolation_input, model.options, model.data_descriptor)
