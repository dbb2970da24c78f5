"""Error bounds of the per-pair phase arithmetic (pyiid_gb300/csrc/
pair_math.cuh), measured on the CPU.

tests/pair_math_host.cpp compiles the header with g++, with the correctly
rounded device intrinsics mapped to the same IEEE operations on the host, so
the values are the device's bit for bit (the seeds' hardware sin/cos is
replaced by the host's; those two figures measure the phase reduction).
Every figure is checked against FP64 truth from the same float32 positions:
r, the float-pair phase step theta = dq r, sin/cos of theta, the fold of
2 theta to theta2 in [-pi/2, pi/2] with sign sigma2, kappa = 2 sin(theta2/2),
the chunk seeds and the half-angle Taylor sin/cos on [-pi/4, pi/4].
"""
import json
import os
import shutil
import subprocess

import pytest

from conftest import REPO

CUDA_INC = '/usr/local/cuda/include'


@pytest.fixture(scope='module')
def errors():
    gxx = shutil.which('g++')
    if gxx is None or not os.path.exists(os.path.join(CUDA_INC,
                                                      'cuda_runtime.h')):
        pytest.skip('needs g++ and the CUDA headers')
    out_dir = os.path.join(REPO, 'tests', '_build')
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, 'pair_math_host')
    subprocess.run([gxx, '-O2', '-std=c++17', '-ffp-contract=off',
                    '-I', CUDA_INC,
                    '-I', os.path.join(REPO, 'pyiid_gb300', 'csrc'),
                    os.path.join(REPO, 'tests', 'pair_math_host.cpp'),
                    '-o', exe], check=True)
    res = subprocess.run([exe, '200000', '1'], check=True,
                         capture_output=True, text=True)
    return json.loads(res.stdout)


def test_distance_and_phase_step(errors):
    # r is the float rounding of sqrt of the float-rounded r^2: 1.5 ulp at
    # most; the phase step carries the low parts (float pair, ~2^-46)
    assert errors['r_rel'] <= 1.0e-7
    assert errors['theta_rel'] <= 1e-12
    assert errors['theta_max'] > 30  # phases up to tens of radians covered


def test_fold_of_the_double_step(errors):
    # theta2 stays in [-pi/2, pi/2] and (sigma2, theta2) reproduce 2 theta
    assert errors['theta2_over_half_pi'] <= 1e-7
    assert errors['half_angle_norm'] <= 3e-7
    assert errors['sin_2theta_abs'] <= 4e-7
    assert errors['cos_2theta_abs'] <= 4e-7
    assert errors['kappa_abs'] == 0.0


def test_quarter_turn_rotation_gives_sin_cos_theta(errors):
    assert errors['sin_theta_abs'] <= 2e-7
    assert errors['cos_theta_abs'] <= 2e-7


def test_taylor_half_angle_within_one_ulp(errors):
    # sin and cos of |x| <= pi/4: below one float ulp of 1 (1.19e-7)
    assert errors['taylor_sin_abs'] <= 1.2e-7
    assert errors['taylor_cos_abs'] <= 1.2e-7


def test_seed_reduction(errors):
    # k0 theta reduced modulo 2 pi as a float pair, k0 < 1500; the odd slot
    # is the even one rotated by theta (two more roundings)
    assert errors['seed_abs'] <= 5e-7
    assert errors['seed_odd_abs'] <= 7e-7
