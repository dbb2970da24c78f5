"""Oracle (test infrastructure only): NumPy restatement of the spring
potentials of pyiid/calc/spring_calc.py, in the reference's precisions
(positions cast to float32, pair vectors d[i, j] = q[j] - q[i] and distances
in float32 as cpu_nxn.get_d_array / get_r_array form them, everything else
float64).  Nothing here runs in the product path.

Functions (reference lines):
  spring_nrg, spring_force              :99-141
  voxel_spring_nrg, atomwise_spring_nrg :145-182
  com_spring_nrg, com_spring_force      :185-217
  voxel_com_spring_nrg, atomwise_com    :220-249
  att_spring_nrg, att_spring_force      :252-295
  voxel_att_spring_nrg, atomwise_att    :298-331
The voxel grids take int(cell diagonal / resolution) voxels per axis (the
reference passes the float quotient to np.zeros, which old numpy truncated).
The reference's atomwise_spring_nrg prints its matrix; that is not restated.
"""
import numpy as np


def _pairs(q):
    q = np.asarray(q, np.float32)
    d = q[None, :, :] - q[:, None, :]          # d[i, j] = q[j] - q[i]
    r = np.sqrt(np.sum(d * d, axis=2, dtype=np.float32)).astype(np.float32)
    return d, r


def _pair_nrg(q, k, rt, att):
    d, r = _pairs(q)
    thresh = np.greater(r, rt) if att else np.less(r, rt)
    np.fill_diagonal(thresh, False)
    mag = np.zeros(r.shape)
    mag[thresh] = k * (r[thresh] - rt)
    return float(np.sum(mag[thresh] / 2. * (r[thresh] - rt)))


def _pair_force(q, k, rt, att):
    d, r = _pairs(q)
    n = len(r)
    thresh = np.greater(r, rt) if att else np.less(r, rt)
    np.fill_diagonal(thresh, False)
    mag = np.zeros(r.shape)
    mag[thresh] = k * (r[thresh] - rt)
    direction = np.zeros((n, n, 3))
    with np.errstate(all='ignore'):
        for tz in range(3):
            direction[thresh, tz] = d[thresh, tz] / r[thresh] * mag[thresh]
    direction[np.isnan(direction)] = 0.0
    return direction.sum(axis=1)


def spring_nrg(q, k, rt):
    return _pair_nrg(q, k, rt, att=False)


def spring_force(q, k, rt):
    return _pair_force(q, k, rt, att=False)


def att_spring_nrg(q, k, rt):
    return _pair_nrg(q, k, rt, att=True)


def att_spring_force(q, k, rt):
    return _pair_force(q, k, rt, att=True)


def _disp(q, com):
    disp = np.asarray(q, np.float32) - np.asarray(com, np.float64)
    return disp, np.sqrt(np.sum(disp ** 2, axis=1))


def com_spring_nrg(q, k, rt, com):
    disp, dist = _disp(q, com)
    thresh = np.greater(dist, rt)
    mag = np.zeros(len(dist))
    mag[thresh] = k * (dist[thresh] - rt)
    return float(np.sum(mag[thresh] / 2. * (dist[thresh] - rt)))


def com_spring_force(q, k, rt, com):
    disp, dist = _disp(q, com)
    thresh = np.greater(dist, rt)
    mag = np.zeros(len(dist))
    mag[thresh] = k * (dist[thresh] - rt)
    direction = np.zeros(disp.shape)
    with np.errstate(all='ignore'):
        for tz in range(3):
            direction[thresh, tz] = disp[thresh, tz] / dist[thresh] * \
                mag[thresh]
    return direction * -1.


def voxel_shape(cell_diagonal, resolution):
    return tuple(int(c / resolution) for c in cell_diagonal)


def _voxel_centres(shape, resolution):
    idx = np.indices(shape).reshape(3, -1).T.astype(np.float64)
    return (idx + .5) * resolution


def voxel_nrg(q, k, rt, sp_type, cell_diagonal, resolution, com=None):
    """voxel_spring_nrg / voxel_att_spring_nrg / voxel_com_spring_nrg."""
    shape = voxel_shape(cell_diagonal, resolution)
    c = _voxel_centres(shape, resolution)
    if sp_type == 'com':
        t = np.sqrt(np.sum((c - np.asarray(com)) ** 2, axis=1))
        e = np.where(t > rt, .5 * k * (t - rt) ** 2, 0.0)
    else:
        qq = np.asarray(q, np.float32).astype(np.float64)
        t = np.sqrt(np.sum((c[:, None, :] - qq[None, :, :]) ** 2, axis=2))
        act = (t > rt) if sp_type == 'att' else (t < rt)
        e = np.where(act, .5 * k * (t - rt) ** 2, 0.0).sum(axis=1)
    return (e * 2).reshape(shape)


def atomwise_nrg(q, k, rt, sp_type, com=None):
    """atomwise_spring_nrg / atomwise_att_spring_nrg / atomwise_com."""
    if sp_type == 'com':
        disp, dist = _disp(q, com)
        nrg = .5 * k * (dist - rt) ** 2
        nrg[np.where(dist < rt)] = 0.0
        return np.sum(nrg, axis=0) * 2
    d, r = _pairs(q)
    nrg = .5 * k * (r - rt) ** 2
    if sp_type == 'att':
        nrg[np.where(r < rt)] = 0.0
    else:
        nrg[np.where(r > rt)] = 0.0
        np.fill_diagonal(nrg, 0.0)
    return -np.sum(nrg, axis=0) * 2
