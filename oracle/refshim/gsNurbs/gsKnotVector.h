// Test-only stand-in for gismo's gsKnotVector, as gsAPALMData uses it: a sorted sequence of
// (possibly repeated) knots with insertion, indexed access, iteration, an affine map onto
// [c, d] and a shift of the knots from a given value on.  This project's own code.
#pragma once

#include <algorithm>
#include <vector>

#include <gsCore/gsLinearAlgebra.h>

namespace gismo {

template <class T = real_t>
class gsKnotVector {
public:
    typedef typename std::vector<T>::const_iterator const_iterator;

    explicit gsKnotVector(int /*degree*/ = -1) {}
    explicit gsKnotVector(const std::vector<T>& knots) : k_(knots) {
        GISMO_ASSERT(std::is_sorted(k_.begin(), k_.end()), "knots must be sorted");
    }

    size_t size() const { return k_.size(); }
    const T& at(size_t i) const { return k_.at(i); }
    const T& operator[](size_t i) const { return k_[i]; }
    const T& first() const { return k_.front(); }
    const T& last() const { return k_.back(); }
    const_iterator begin() const { return k_.begin(); }
    const_iterator end() const { return k_.end(); }

    // insert one knot after any equal ones
    void insert(T knot) { k_.insert(std::upper_bound(k_.begin(), k_.end(), knot), knot); }
    // affine map of every knot onto [c, d]
    void transform(T c, T d) {
        const T a = k_.front(), s = (d - c) / (k_.back() - a);
        for (T& v : k_) v = c + (v - a) * s;
    }
    // add `amount` to every knot at or above `start`
    void addConstant(T start, T amount) {
        for (T& v : k_)
            if (v >= start) v += amount;
    }
    gsMatrix<T> asMatrix() const {
        gsMatrix<T> m(1, (index_t)k_.size());
        for (size_t i = 0; i < k_.size(); ++i) m(0, (index_t)i) = k_[i];
        return m;
    }

private:
    std::vector<T> k_;
};

}  // namespace gismo
