"""Names the reference's jit_extensions module imports; inert on CPU."""
void = None
