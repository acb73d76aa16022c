"""Empty stand-in for ``pyopencl.tools`` (imported, never used, by the reference)."""
