"""The autotuner's cache on the CPU (device name and context faked): keys
bucket the atom count by powers of two and separate kernels, bin counts,
species counts and devices; the JSON file survives a round trip and is
written atomically; apply_cached sets exactly the cached variants."""
import os

import pytest

from conftest import REPO


@pytest.fixture
def tune(monkeypatch):
    from pyiid_gb300 import autotune
    path = os.path.join(REPO, 'tests', '_build', 'tuning_cache.json')
    os.makedirs(os.path.dirname(path), exist_ok=True)
    if os.path.exists(path):
        os.remove(path)
    monkeypatch.setenv('PYIID_GB300_TUNE_CACHE', path)
    monkeypatch.setattr(autotune.torch.cuda, 'get_device_name',
                        lambda *a: 'NVIDIA GB300')
    return autotune


def test_keys_bucket_atoms_and_separate_problems(tune):
    k = tune._key
    assert k('fq', 1000, 500, 1) == k('fq', 513, 500, 1)     # N <= 1024
    assert k('fq', 1000, 500, 1) != k('fq', 1025, 500, 1)
    assert k('fq', 1000, 500, 1) != k('grad_fq', 1000, 500, 1)
    assert k('fq', 1000, 500, 1) != k('fq', 1000, 498, 1)
    assert k('fq', 1000, 500, 1) != k('fq', 1000, 500, 2)
    assert k('fq', 0, 500, 1) == k('fq', 1, 500, 1)
    assert k('fq', 1000, 500, 1).startswith('NVIDIA GB300|')


def test_cache_round_trip_and_apply(tune, monkeypatch):
    assert tune._load_cache() == {}
    c = {tune._key('fq', 20000, 1475, 1): 23,
         tune._key('grad_fq', 20000, 1475, 1): 3}
    tune._save_cache(c)
    assert tune._load_cache() == c
    assert not any(f.startswith('tuning_cache.json.')
                   for f in os.listdir(os.path.dirname(tune.cache_path())))

    class FakeCtx:
        def __init__(self):
            self.set = {}

        def set_variant(self, kernel, v):
            self.set[kernel] = v

    ctx = FakeCtx()
    monkeypatch.setattr(tune, 'context', lambda device=None: ctx)
    assert tune.apply_cached(20000, 1475, 1) == {'fq': 23, 'grad_fq': 3}
    assert ctx.set == {'fq': 23, 'grad_fq': 3}
    ctx.set.clear()
    assert tune.apply_cached(20000, 1500, 1) == {} and ctx.set == {}


def test_unreadable_cache_is_empty(tune):
    with open(tune.cache_path(), 'w') as f:
        f.write('{not json')
    assert tune._load_cache() == {}
