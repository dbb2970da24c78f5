"""GB300-native (sm_103a) implementation of pyIID's elastic-scattering path.

Layers (bottom up):
  * ``include/pyiid_gb300.h`` / ``pyiid_gb300/csrc`` -- the C ABI and the
    hand-written CUDA kernels (Debye pair sums, adjoint, G(r) transform);
  * :mod:`pyiid_gb300.debye` -- torch-tensor functional API over the C ABI;
  * :mod:`pyiid_gb300.experiments.elasticscatter` -- drop-in ``ElasticScatter``
    with the 'GB300' processor; :mod:`pyiid_gb300.calc` -- ``Calc1D`` /
    ``PDFCalc`` / ``FQCalc``; :mod:`pyiid_gb300.sim` -- the samplers.
"""
__version__ = '1.0.0'
