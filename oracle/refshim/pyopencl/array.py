"""Empty stand-in for ``pyopencl.array`` (imported, never used, by the reference)."""
