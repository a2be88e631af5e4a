/* sse_shim.h -- forced include for compiling the reference's SSE voxtrees
 * sources (SSE_INTRIN on, x86 only) with gcc, for the layout test fixtures.
 *
 * TEST INFRASTRUCTURE ONLY.  The reference is written for clang, which
 * converts the __m128i result of _mm_set_epi32 / _mm_set1_epi32 to __m128
 * implicitly (src/voxtrees/geom-sse.c:7,56); gcc refuses.  These wrappers
 * reinterpret the integer vector as float lanes, which is what clang does. */
#ifndef VOX_SSE_SHIM_H
#define VOX_SSE_SHIM_H
#include <smmintrin.h>
#define _mm_set_epi32(a, b, c, d) ((__m128)_mm_set_epi32((a), (b), (c), (d)))
#define _mm_set1_epi32(a) ((__m128)_mm_set1_epi32((a)))
#endif
