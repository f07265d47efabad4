// Matrix.h -- host matrix / vector containers of the sqaod C++ solver API.
//
// Interface of sqaodc/common/Matrix.h: MatrixType<V> (rows, cols, stride,
// data; owning or mapping external memory), VectorType<V> (size, data),
// BitSet = VectorType<char>, BitSetArray, BitSetPair, BitSetPairArray,
// BitMatrix.  Rows here are dense (stride == cols) unless memory is mapped
// with an explicit stride.
#pragma once

#include <string.h>

#include <utility>

#include <sqaodc/common/Array.h>
#include <sqaodc/common/types.h>

namespace sqaod {

template <class V>
struct MatrixType {
    typedef V ValueType;

    MatrixType() : data(nullptr), rows(0), cols(0), stride(0), mapped(false) {}
    MatrixType(SizeType r, SizeType c) : MatrixType() { allocate(r, c); }
    explicit MatrixType(const Dim &d) : MatrixType(d.rows, d.cols) {}
    MatrixType(const MatrixType &o) : MatrixType() { copyFrom(o); }
    MatrixType(MatrixType &&o) noexcept : MatrixType() { moveFrom(o); }
    // maps external memory (not owned)
    MatrixType(V *d, SizeType r, SizeType c, SizeType s) : data(d), rows(r), cols(c), stride(s), mapped(true) {}
    virtual ~MatrixType() { free(); }

    MatrixType &operator=(const MatrixType &o) {
        if (this != &o) copyFrom(o);
        return *this;
    }
    MatrixType &operator=(MatrixType &&o) noexcept {
        if (this != &o) moveFrom(o);
        return *this;
    }

    Dim dim() const { return Dim(rows, cols); }
    void map(V *d, SizeType r, SizeType c, SizeType s) {
        free();
        data = d; rows = r; cols = c; stride = s; mapped = true;
    }
    void allocate(SizeType r, SizeType c) {
        free();
        rows = r; cols = c; stride = c; mapped = false;
        data = (r > 0 && c > 0) ? new V[(size_t)r * c]() : nullptr;
    }
    void resize(SizeType r, SizeType c) {
        if (r != rows || c != cols || mapped) allocate(r, c);
    }
    void resize(const Dim &d) { resize(d.rows, d.cols); }
    void free() {
        if (!mapped) delete[] data;
        data = nullptr; rows = cols = stride = 0; mapped = false;
    }
    void copyFrom(const MatrixType &src) {
        if (mapped && rows == src.rows && cols == src.cols) {
            for (SizeType r = 0; r < rows; ++r) memcpy(rowPtr(r), src.rowPtr(r), sizeof(V) * cols);
            return;
        }
        allocate(src.rows, src.cols);
        for (SizeType r = 0; r < rows; ++r) memcpy(rowPtr(r), src.rowPtr(r), sizeof(V) * cols);
    }
    void moveFrom(MatrixType &src) {
        free();
        data = src.data; rows = src.rows; cols = src.cols; stride = src.stride; mapped = src.mapped;
        src.data = nullptr; src.rows = src.cols = src.stride = 0; src.mapped = false;
    }
    void fill(const V &v) {
        for (SizeType r = 0; r < rows; ++r)
            for (SizeType c = 0; c < cols; ++c) (*this)(r, c) = v;
    }

    V &operator()(IdxType r, IdxType c) { return data[(size_t)r * stride + c]; }
    const V &operator()(IdxType r, IdxType c) const { return data[(size_t)r * stride + c]; }
    V *rowPtr(IdxType r) { return data + (size_t)r * stride; }
    const V *rowPtr(IdxType r) const { return data + (size_t)r * stride; }

    V *data;
    SizeType rows, cols, stride;
    bool mapped;
};

template <class V>
struct VectorType {
    typedef V ValueType;

    VectorType() : data(nullptr), size(0), mapped(false) {}
    explicit VectorType(SizeType n) : VectorType() { allocate(n); }
    VectorType(const VectorType &o) : VectorType() { copyFrom(o); }
    VectorType(VectorType &&o) noexcept : VectorType() { moveFrom(o); }
    VectorType(V *d, SizeType n) : data(d), size(n), mapped(true) {}
    virtual ~VectorType() { free(); }

    VectorType &operator=(const VectorType &o) {
        if (this != &o) copyFrom(o);
        return *this;
    }
    VectorType &operator=(VectorType &&o) noexcept {
        if (this != &o) moveFrom(o);
        return *this;
    }
    // fills every element (the reference's scalar assignment)
    VectorType &operator=(const V &v) {
        for (SizeType i = 0; i < size; ++i) data[i] = v;
        return *this;
    }

    void map(V *d, SizeType n) {
        free();
        data = d; size = n; mapped = true;
    }
    void allocate(SizeType n) {
        free();
        size = n; mapped = false;
        data = n ? new V[n]() : nullptr;
    }
    void resize(SizeType n) {
        if (n != size || mapped) allocate(n);
    }
    void free() {
        if (!mapped) delete[] data;
        data = nullptr; size = 0; mapped = false;
    }
    void copyFrom(const VectorType &src) {
        if (!(mapped && size == src.size)) allocate(src.size);
        if (size) memcpy(data, src.data, sizeof(V) * size);
    }
    void moveFrom(VectorType &src) {
        free();
        data = src.data; size = src.size; mapped = src.mapped;
        src.data = nullptr; src.size = 0; src.mapped = false;
    }
    V sum() const {
        V s = V();
        for (SizeType i = 0; i < size; ++i) s += data[i];
        return s;
    }

    V &operator()(IdxType i) { return data[i]; }
    const V &operator()(IdxType i) const { return data[i]; }

    friend bool operator==(const VectorType &a, const VectorType &b) {
        return a.size == b.size && (a.size == 0 || memcmp(a.data, b.data, sizeof(V) * a.size) == 0);
    }
    friend bool operator!=(const VectorType &a, const VectorType &b) { return !(a == b); }

    V *data;
    SizeType size;
    bool mapped;
};

typedef VectorType<char> BitSet;
typedef ArrayType<BitSet> BitSetArray;
typedef MatrixType<char> BitMatrix;

struct BitSetPair {
    BitSetPair() {}
    BitSetPair(const BitSet &b0, const BitSet &b1) : bits0(b0), bits1(b1) {}
    BitSet bits0, bits1;
    friend bool operator==(const BitSetPair &a, const BitSetPair &b) { return a.bits0 == b.bits0 && a.bits1 == b.bits1; }
    friend bool operator!=(const BitSetPair &a, const BitSetPair &b) { return !(a == b); }
};
typedef ArrayType<BitSetPair> BitSetPairArray;

}  // namespace sqaod
