// Common.h -- umbrella header and helpers of the sqaod C++ solver API
// (sqaodc/common/Common.h of the reference: bit-set sequences, unpacking,
// symmetry check, x <-> q conversion, errors).
#pragma once

#include <stdexcept>

#include <sqaodc/common/Array.h>
#include <sqaodc/common/Matrix.h>
#include <sqaodc/common/Preference.h>
#include <sqaodc/common/Solver.h>
#include <sqaodc/common/types.h>

#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

namespace sqaod {

// rows of bits (MSB-first) of the packed values [bBegin, bEnd)
template <class V>
void createBitSetSequence(V *bits, SizeType stride, SizeType nBits, PackedBitSet bBegin, PackedBitSet bEnd) {
    for (PackedBitSet b = bBegin; b < bEnd; ++b, bits += stride)
        for (int pos = 0; pos < nBits; ++pos) bits[pos] = V((b >> (nBits - 1 - pos)) & 1);
}

void unpackBitSet(BitSet *unpacked, PackedBitSet packed, int N);

// exact W == W^T of an n x n row-major matrix with row stride ld, compared in
// 64 x 64 tiles so that the transposed reads stay in cache
template <class real>
bool isSymmetric(const real *W, size_t n, size_t ld) {
    const size_t B = 64;
    for (size_t r0 = 0; r0 < n; r0 += B)
        for (size_t c0 = 0; c0 <= r0; c0 += B)
            for (size_t r = r0; r < r0 + B && r < n; ++r)
                for (size_t c = c0; c < c0 + B && c < r; ++c)
                    if (W[r * ld + c] != W[c * ld + r]) return false;
    return true;
}

template <class real>
bool isSymmetric(const MatrixType<real> &W) {
    if (W.rows != W.cols) return false;
    return isSymmetric(W.data, (size_t)W.rows, (size_t)W.stride);
}

// x = (q + 1) / 2
BitSet x_from_q(const BitSet &q);

// std::runtime_error with a printf-style message (the reference's throwErrorIf)
[[noreturn]] void throwError(const char *fmt, ...);
void log(const char *fmt, ...);

}  // namespace sqaod

#define throwErrorIf(cond, ...) \
    do {                        \
        if (cond) ::sqaod::throwError(__VA_ARGS__); \
    } while (0)

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#include <sqaodc/common/Formulas.h>
