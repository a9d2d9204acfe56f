def __getattr__(n):
    raise AttributeError(f"plotting is not available in the jax stand-in ({n})")
