// Array.h -- growable array of the sqaod C++ solver API
// (interface of sqaodc/common/Array.h: ArrayType<V> with size(), pushBack(),
// insert(), clear(), iterators; the storage here is a std::vector).
#pragma once

#include <vector>

#include <sqaodc/common/types.h>

namespace sqaod {

template <class V>
struct ArrayType {
    typedef V *iterator;
    typedef const V *const_iterator;
    typedef V ValueType;

    ArrayType() {}
    explicit ArrayType(SizeType capacity) { v_.reserve(capacity); }

    SizeType size() const { return (SizeType)v_.size(); }
    SizeType capacity() const { return (SizeType)v_.capacity(); }
    bool empty() const { return v_.empty(); }
    void reserve(SizeType n) { v_.reserve(n); }
    void clear() { v_.clear(); }
    void pushBack(const V &v) { v_.push_back(v); }
    void pushBack(V &&v) { v_.push_back(static_cast<V &&>(v)); }
    void erase(SizeType idx) { v_.erase(v_.begin() + idx); }
    template <class It>
    void insert(It first, It last) {
        v_.insert(v_.end(), first, last);
    }

    V *data() { return v_.data(); }
    const V *data() const { return v_.data(); }
    iterator begin() { return v_.data(); }
    iterator end() { return v_.data() + v_.size(); }
    const_iterator begin() const { return v_.data(); }
    const_iterator end() const { return v_.data() + v_.size(); }
    V &operator[](IdxType idx) { return v_[idx]; }
    const V &operator[](IdxType idx) const { return v_[idx]; }

    friend bool operator==(const ArrayType &a, const ArrayType &b) { return a.v_ == b.v_; }
    friend bool operator!=(const ArrayType &a, const ArrayType &b) { return !(a == b); }

private:
    std::vector<V> v_;
};

typedef ArrayType<PackedBitSet> PackedBitSetArray;
typedef ArrayType<PackedBitSetPair> PackedBitSetPairArray;

inline bool operator==(const PackedBitSetPair &a, const PackedBitSetPair &b) {
    return a.bits0 == b.bits0 && a.bits1 == b.bits1;
}

}  // namespace sqaod
