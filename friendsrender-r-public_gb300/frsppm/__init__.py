"""Python side of the GB300 SPPM renderer: scene generators, scene file I/O,
the in-tree build and the ctypes binding of the C-ABI (include/friendsrender.h).
The renderer itself is the native library libfrsppm.so."""
