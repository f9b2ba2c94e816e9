// dt::vector<Size>: a host array of Size doubles with the reference's
// interface (src/dt/vector.h:33-165): element access, iterators, + - * /, the
// dot product as operator*, and abs() as the RMS norm sqrt(sum e^2)/sqrt(Size).
// The GPU shim keeps fields in these host arrays between calls and moves them
// through the C ABI, which accepts host pointers.
#ifndef DT_VECTOR_H
#define DT_VECTOR_H

#include <cassert>
#include <cmath>
#include <cstring>
#include <initializer_list>
#include <ostream>
#include <vector>

namespace dt {

template <unsigned int Size>
class vector {
  private:
    typedef std::vector<double> vector_type;

  public:
    typedef typename vector_type::value_type value_type;
    typedef typename vector_type::iterator iterator;
    typedef typename vector_type::const_iterator const_iterator;
    typedef typename vector_type::reference reference;
    typedef typename vector_type::const_reference const_reference;
    typedef typename vector_type::pointer pointer;
    typedef typename vector_type::const_pointer const_pointer;
    typedef typename vector_type::size_type size_type;

  protected:
    vector_type values;

  public:
    vector(const vector<Size>& v) : values(v.values) {}
    vector(double value = 0.0) : values(Size, value) {}
    vector(std::initializer_list<value_type> v) : values(v) { assert(v.size() == Size); }
    virtual ~vector() {}

    vector<Size>& operator=(const vector<Size>& o) {
        values = o.values;
        return *this;
    }
    vector<Size>& operator=(std::initializer_list<value_type> v) {
        assert(v.size() == Size);
        values = v;
        return *this;
    }

    reference operator[](unsigned int i) { return values[i]; }
    const_reference operator[](unsigned int i) const { return values[i]; }
    size_type size() const { return Size; }
    iterator begin() { return values.begin(); }
    iterator end() { return values.end(); }
    const_iterator begin() const { return values.begin(); }
    const_iterator end() const { return values.end(); }
    const_iterator cbegin() const { return values.cbegin(); }
    const_iterator cend() const { return values.cend(); }
    pointer data() { return values.data(); }
    const_pointer data() const { return values.data(); }

    // dot product
    value_type operator*(const vector<Size>& o) const {
        value_type r = 0.0;
        for (unsigned i = 0; i < Size; ++i) r += values[i] * o.values[i];
        return r;
    }
    vector<Size>& operator+=(const vector<Size>& o) {
        for (unsigned i = 0; i < Size; ++i) values[i] += o.values[i];
        return *this;
    }
    vector<Size>& operator-=(const vector<Size>& o) {
        for (unsigned i = 0; i < Size; ++i) values[i] -= o.values[i];
        return *this;
    }
    vector<Size>& operator*=(double c) {
        for (auto& v : values) v *= c;
        return *this;
    }
    vector<Size>& operator/=(double c) {
        for (auto& v : values) v /= c;
        return *this;
    }
};

// RMS norm
template <unsigned int Size>
double abs(const vector<Size>& v) {
    double m = 0.0;
    for (auto it = v.cbegin(); it != v.cend(); ++it) m += (*it) * (*it);
    return std::sqrt(m) / std::sqrt((double)Size);
}

template <unsigned int Size>
vector<Size> operator+(vector<Size> l, const vector<Size>& r) { return l += r; }
template <unsigned int Size>
vector<Size> operator-(vector<Size> l, const vector<Size>& r) { return l -= r; }
template <unsigned int Size>
vector<Size> operator*(double c, vector<Size> v) { return v *= c; }
template <unsigned int Size>
vector<Size> operator/(vector<Size> v, double c) { return v /= c; }

template <unsigned int Size>
std::ostream& operator<<(std::ostream& out, const vector<Size>& v) {
    bool sep = false;
    out << "[";
    for (auto it = v.cbegin(); it != v.cend(); ++it) {
        if (sep) out << ", ";
        sep = true;
        out << *it;
    }
    return out << "]'";
}

}  // namespace dt

#endif
