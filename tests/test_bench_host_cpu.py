"""bench.py's host-side helpers, which fill fields of its JSON line: the
clock summary of the nvidia-smi samples (median SM clock under load,
throttle reasons), the DRAM traffic read from the committed ncu summary,
the workload and its config block, the bounded CPU sample and the line of
the reference arm (--impl reference)."""
import os

import numpy as np

from conftest import REPO


def _sampler(tmp_lines):
    import bench
    s = bench.ClockSampler(0)
    os.makedirs(os.path.join(REPO, 'tests', '_build'), exist_ok=True)
    s.path = os.path.join(REPO, 'tests', '_build', 'clocks_sample.csv')
    with open(s.path, 'w') as f:
        f.write('\n'.join(tmp_lines) + '\n')
    s.proc = object()  # as if nvidia-smi had been started
    return s


def test_clock_summary_under_load_and_reasons():
    idle = '1980, 2070, 150.0, 0x0, Not Active, Not Active, Not Active, ' \
           'Not Active'
    busy = '2070, 2070, 900.0, 0x0, Not Active, Not Active, Not Active, ' \
           'Not Active'
    capped = '1950, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, ' \
             'Active'
    s = _sampler([idle, busy, busy, capped, 'garbage line', '1, 2, x, 4'])
    out = s.summary()
    # samples below half the peak power are not "under load"
    assert out['sm_mhz'] == 2070.0
    assert out['sm_max_mhz'] == 2070.0
    assert out['power_w_max'] == 1390.0
    assert out['samples'] == 4
    assert out['reasons'] == ['sw_power_cap']
    hot = '1500, 2070, 1000.0, 0x40, Not Active, Active, Not Active, ' \
          'Not Active'
    assert _sampler([hot]).summary()['reasons'] == ['hw_thermal_slowdown']


def test_clock_summary_without_samples():
    import bench
    s = bench.ClockSampler(0)
    assert s.summary()['reasons'] == ['unavailable']
    assert _sampler(['nothing useful']).summary()['reasons'] == ['no samples']


def test_traffic_comes_from_the_committed_profile():
    import bench
    t = bench.traffic_from_profile('fqgrad2_kernel')
    assert t is not None and 3.0e8 < t < 4.0e8   # ~332 MB per launch
    assert bench.traffic_from_profile('gradfq2_kernel') is not None
    assert bench.traffic_from_profile('no_such_kernel') is None


def test_workload_and_config_block():
    import bench
    pos, sp, tab, n_bins, k_begin = bench.workload(2000)
    assert pos.shape == (2000, 3) and pos.dtype == np.float32
    assert n_bins == 1500 and k_begin == 25          # Q 0.5-30 step 0.02
    assert sp.shape == (2000,) and tab.shape == (1, 1500)
    c = bench.config_dict(1500, 25)
    assert c['n_atoms'] == 20000 and c['bins_returned'] == 1475
    assert c['pairs'] == 20000 * 19999 // 2
    assert c == bench.config_dict(1500, 25, 20000)
    assert 'flushed' in c['l2']
    assert bench.measured_hbm_gbs() is None or bench.measured_hbm_gbs() > 1000


def test_cpu_sample_reports_a_bounded_port_measurement():
    import bench
    out = bench.cpu_sample(target_s=0.2, threads=2, n_atoms=300)
    assert out['kind'] == 'port' and out['unit'] == 'evals/s'
    assert out['cores'] == 2 and out['value'] > 0
    assert 'of 44850 pairs' in out['sample'] and out['seconds'] > 0
    assert out['extrapolated'] is True and out['pairs_per_evaluation'] == 44850


def test_full_cpu_evaluations_are_measured_not_scaled():
    import bench
    out = bench.cpu_full_evaluations(sizes=(120,), threads=2)['n120']
    assert out['extrapolated'] is False and out['pairs'] == 120 * 119 // 2
    assert out['seconds_per_eval'] > 0 and out['cores'] == 2
    assert out['scaled_by_pairs_to_workload_evals_per_s'] < out['evals_per_s']


def test_reference_arm_line_follows_the_contract(monkeypatch):
    """--impl reference: the reference's CPU path (the port here) on the
    same metric, config and units, with a cpu_baseline and an e2e block
    that moves no bytes; rank > 0 prints nothing."""
    import types
    import bench
    samples = iter([0.5, 0.7])

    def fake_sample(target_s=15.0, threads=0, n_atoms=None):
        return {'value': next(samples), 'unit': 'evals/s', 'cores': 8,
                'kind': 'port', 'sample': 'stub', 'seconds': 1.0,
                'extrapolated': True, 'pairs_timed': 1000,
                'pairs_per_evaluation': 199990000}
    monkeypatch.setattr(bench, 'cpu_sample', fake_sample)
    monkeypatch.setattr(bench, 'cpu_full_evaluations',
                        lambda: {'n1000': {'extrapolated': False}})
    args = types.SimpleNamespace(steps=2, warmup=0)
    assert bench.run_reference(args, 1, 2) is None
    line = bench.run_reference(args, 0, 1)
    assert line['impl'] == 'reference' and line['metric'] == bench.METRIC
    assert abs(line['value'] - 0.6) < 1e-12
    assert line['unit'] == 'evals/s' and line['higher_is_better'] is True
    assert line['cpu_baseline']['value'] == line['value']
    assert line['cpu_baseline']['kind'] == 'port'
    assert line['e2e'] == {'value': line['value'], 'unit': 'evals/s',
                           'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}
    assert line['config']['bins_returned'] == 1475
    # the reader sees what was timed and what was scaled
    assert line['extrapolated'] is True
    assert line['timed']['pairs_per_step'] == 1000
    assert line['ms_per_step'] == 1000.0
    assert line['measured_full_evaluations']['n1000']['extrapolated'] is False
    # both arms share one config block
    assert line['config'] == bench.config_dict(1500, 25)


def test_ess_estimator_on_known_processes():
    """Geyer's initial positive sequence: white noise keeps about T samples
    per chain, an AR(1) chain with rho = 0.9 about T (1 - rho) / (1 + rho)."""
    import bench
    rng = np.random.default_rng(0)
    T, B = 4000, 4
    w = rng.normal(size=(T, B))
    assert 0.8 * T < bench.ess_sum(w) / B < 1.2 * T
    x = np.zeros((T, B))
    for t in range(1, T):
        x[t] = 0.9 * x[t - 1] + rng.normal(size=B)
    want = T * 0.1 / 1.9
    assert 0.7 * want < bench.ess_sum(x) / B < 1.3 * want
    assert bench.ess_sum(np.ones((10, 2))) == 0.0


def test_variant_option_rejects_unknown_kernels_before_device_work():
    """--variant KERNEL=INDEX names a launch-variant slot of the library;
    anything else ends with a usage error (exit 2) before a context is
    created, so no device is touched."""
    import subprocess
    import sys
    for bad in ('nosuch=1', 'mlp', 'mlp=x'):
        r = subprocess.run([sys.executable, os.path.join(REPO, 'bench.py'),
                            '--only-workload', 'surrogate_forces_au1000x64',
                            '--variant', bad],
                           capture_output=True, text=True, timeout=300)
        assert r.returncode == 2, (bad, r.returncode, r.stderr[-400:])
        assert '--variant' in r.stderr
