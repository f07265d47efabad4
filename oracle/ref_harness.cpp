// ref_harness.cpp -- exposes the reference's own MT19937 (sqaodc/common/Random.cpp)
// and AVX2 dot product (sqaodc/cpu/Dot_SIMD.cpp), compiled from the reference
// sources by oracle/build.py into oracle/_ref/libsqaod_ref.so, through a plain
// C interface, so that tests can pin the oracle's restatements against them.
// Test infrastructure only; this file contains no reference code.
#include <sqaodc/common/Random.h>
#include <sqaodc/cpu/Dot_SIMD.h>
#include <stdint.h>

extern "C" {

// first n words of sqaod::Random after seed(s)
void ref_mt_stream(unsigned long long s, int n, uint32_t *out) {
    sqaod::Random r;
    r.seed(s);
    for (int i = 0; i < n; ++i)
        out[i] = (uint32_t)r.randInt32();
}

// first n random<float>() values after seed(s)
void ref_mt_f32_stream(unsigned long long s, int n, float *out) {
    sqaod::Random r;
    r.seed(s);
    for (int i = 0; i < n; ++i)
        out[i] = r.random<float>();
}

// first n randInt(k) values after seed(s)
void ref_mt_randint_stream(unsigned long long s, int k, int n, int *out) {
    sqaod::Random r;
    r.seed(s);
    for (int i = 0; i < n; ++i)
        out[i] = (int)r.randInt(k);
}

// dot_avx2 over 64-byte aligned, zero-padded copies of the inputs
float ref_dot_avx2(const float *a, const float *b, int N) {
    int padded = (N + 15) / 16 * 16;
    float *pa = (float *)sqaod::aligned_alloc(64, sizeof(float) * padded);
    float *pb = (float *)sqaod::aligned_alloc(64, sizeof(float) * padded);
    for (int i = 0; i < padded; ++i) {
        pa[i] = i < N ? a[i] : 0.f;
        pb[i] = i < N ? b[i] : 0.f;
    }
    float r = sqaod_cpu::dot_avx2(pa, pb, N);
    sqaod::aligned_free(pa);
    sqaod::aligned_free(pb);
    return r;
}

}
