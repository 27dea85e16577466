"""Global mode of the NumPy-backed JAX stand-in (``jax_enable_x64``)."""

X64 = False
