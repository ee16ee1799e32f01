"""Names the reference's jit_extensions module patches; inert on CPU."""
