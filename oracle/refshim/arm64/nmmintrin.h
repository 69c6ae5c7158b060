// Empty stand-in for the x86-only <nmmintrin.h> that the reference includes
// from grid_sse42.h:4.  Only a declaration there names SSE; no SSE code of the
// reference is compiled into the oracle, so non-x86 hosts need no intrinsics.
