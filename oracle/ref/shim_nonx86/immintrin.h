/* Empty stand-in used only on non-x86 hosts: the reference tinysimd headers include
 * <immintrin.h> unconditionally but only use it under __AVX2__/__SSE2__ guards, so
 * on aarch64 the scalar (width 1) path is selected and nothing from here is needed. */
