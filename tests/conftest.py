import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built extension")
    config.addinivalue_line("markers", "slow: longer CPU case")


GOLDEN = os.path.join(ROOT, "tests", "golden")


def load_golden(name):
    import json
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        return json.load(f)


def golden_names():
    return sorted(f[:-5] for f in os.listdir(GOLDEN) if f.endswith(".json"))


_INPUT_CACHE = {}


def golden_inputs(fx):
    """Inputs of a fixture, regenerated from its seed (cached per session)."""
    from atrip_gb300 import synth
    key = (fx["No"], fx["Nv"], fx["seed"], fx["with_j"], fx.get("field", "real"),
           fx.get("eps_imag", 0.0))
    if key not in _INPUT_CACHE:
        if len(_INPUT_CACHE) > 4:
            _INPUT_CACHE.clear()
        _INPUT_CACHE[key] = synth.make_inputs(*key[:3], with_j=key[3], field=key[4],
                                              eps_imag=key[5])
    return _INPUT_CACHE[key]
