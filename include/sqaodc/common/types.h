// types.h -- primitive types of the sqaod C++ solver API
// (same names and meaning as sqaodc/common/types.h:10-27 of the reference).
#pragma once

#include <stddef.h>

namespace sqaod {

typedef int SizeType;
typedef int IdxType;

// packed bit set: variable i of an N-bit problem is bit (N - 1 - i)
typedef unsigned long long PackedBitSet;

struct PackedBitSetPair {
    PackedBitSetPair() : bits0(0), bits1(0) {}
    PackedBitSetPair(PackedBitSet b0, PackedBitSet b1) : bits0(b0), bits1(b1) {}
    PackedBitSet bits0;
    PackedBitSet bits1;
};

struct Dim {
    Dim() : rows(-1), cols(-1) {}
    Dim(SizeType r, SizeType c) : rows(r), cols(c) {}
    Dim transpose() const { return Dim(cols, rows); }
    SizeType rows, cols;
    friend bool operator==(const Dim &a, const Dim &b) { return a.rows == b.rows && a.cols == b.cols; }
    friend bool operator!=(const Dim &a, const Dim &b) { return !(a == b); }
};

// base of every public object; deleted through sqaod::deleteInstance()
struct NullBase {
    virtual ~NullBase() {}
};

template <class V>
inline V divru(V v, int base) {
    return (v + base - 1) / base;
}

template <class V>
inline V roundUp(V v, int base) {
    return divru(v, base) * base;
}

}  // namespace sqaod

#define WAR_VC_NOTHROW
