"""Experiments: elastic scattering (the GB300 processor) lives here, in the
same module path as the reference (pyiid/experiments/elasticscatter)."""
