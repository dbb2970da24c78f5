"""Reference-named helpers of the scattering path (GPU-backed)."""
