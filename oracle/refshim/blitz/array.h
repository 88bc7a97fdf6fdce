/*
 * Minimal stand-in for the Blitz++ array header -- TEST INFRASTRUCTURE ONLY.
 *
 * It exists so that the reference Impec2D sources (which include "blitz/array.h" through
 * src/GenSimDefs.h:23) compile unchanged into oracle/_ref, the reference build that pins the
 * CPU oracle.  Only the Blitz features those sources use are provided, with Blitz's
 * semantics for them:
 *   - Array<T,N>, N = 1..3, C (row-major) storage, last index fastest;
 *   - copy construction shares the data (Blitz reference semantics); copy() makes a deep copy;
 *   - assignment from an array or an expression copies elements index by index;
 *   - resize(), reindexSelf() (move the index base), reverseSelf() (mirror one dimension);
 *   - base(), extent(), shape(), lbound(), ubound(), numElements();
 *   - element access a(i,j[,k]) and a(TinyVector);
 *   - elementwise +, -, *, / between arrays and with scalars (results take the left
 *     operand's index base), and the matching compound assignments;
 *   - the full reductions max(a), min(a), sum(a).
 * Like the real header it brings in <cmath> and <limits>, on which the reference relies.
 * Newly resized storage is zero-filled (Blitz leaves it unspecified; every reference use
 * assigns before reading).
 */
#ifndef IMPEC_REFSHIM_BLITZ_ARRAY_H
#define IMPEC_REFSHIM_BLITZ_ARRAY_H

#include <cmath>
#include <cstddef>
#include <limits>
#include <memory>
#include <ostream>

namespace blitz {

template <typename T, int N>
struct TinyVector {
    T v[N];
    TinyVector() {
        for (int d = 0; d < N; ++d) v[d] = T();
    }
    explicit TinyVector(T a) {
        for (int d = 0; d < N; ++d) v[d] = a;
    }
    TinyVector(T a, T b) {
        static_assert(N == 2, "two components");
        v[0] = a;
        v[1] = b;
    }
    TinyVector(T a, T b, T c) {
        static_assert(N == 3, "three components");
        v[0] = a;
        v[1] = b;
        v[2] = c;
    }
    T& operator[](int d) { return v[d]; }
    const T& operator[](int d) const { return v[d]; }
    T& operator()(int d) { return v[d]; }
    const T& operator()(int d) const { return v[d]; }
    int length() const { return N; }
};

template <typename T, int N>
class Array {
public:
    typedef T T_numtype;

    Array() {}
    explicit Array(int e0) { init1(e0); }
    Array(int e0, int e1) { init2(e0, e1); }
    Array(int e0, int e1, int e2) { init3(e0, e1, e2); }
    explicit Array(const TinyVector<int, N>& e) { allocate(e.v); }
    // Blitz copy construction: a new view of the same data.
    Array(const Array& o) = default;

    // --- shape ---------------------------------------------------------------------
    void resize(int e0) { init1(e0); }
    void resize(int e0, int e1) { init2(e0, e1); }
    void resize(int e0, int e1, int e2) { init3(e0, e1, e2); }
    void resize(const TinyVector<int, N>& e) { allocate(e.v); }
    void reindexSelf(const TinyVector<int, N>& b) {
        for (int d = 0; d < N; ++d) base_[d] = b[d];
    }
    // After reverseSelf(d), index i along d reads what lbound(d)+ubound(d)-i read before.
    void reverseSelf(int d) {
        first_ += (ptrdiff_t)(ext_[d] - 1) * stride_[d];
        stride_[d] = -stride_[d];
    }
    TinyVector<int, N> base() const {
        TinyVector<int, N> r;
        for (int d = 0; d < N; ++d) r[d] = base_[d];
        return r;
    }
    int base(int d) const { return base_[d]; }
    TinyVector<int, N> extent() const {
        TinyVector<int, N> r;
        for (int d = 0; d < N; ++d) r[d] = ext_[d];
        return r;
    }
    int extent(int d) const { return ext_[d]; }
    TinyVector<int, N> shape() const { return extent(); }
    int lbound(int d) const { return base_[d]; }
    int ubound(int d) const { return base_[d] + ext_[d] - 1; }
    int rows() const { return ext_[0]; }
    int cols() const { return ext_[1]; }
    size_t numElements() const {
        size_t n = 1;
        for (int d = 0; d < N; ++d) n *= (size_t)ext_[d];
        return n;
    }
    size_t size() const { return numElements(); }
    T* data() { return first_; }
    const T* data() const { return first_; }
    T* dataFirst() { return first_; }
    const T* dataFirst() const { return first_; }

    // --- element access -------------------------------------------------------------
    T& operator()(int i) { return first_[off(i)]; }
    const T& operator()(int i) const { return first_[off(i)]; }
    T& operator()(int i, int j) { return first_[off(i, j)]; }
    const T& operator()(int i, int j) const { return first_[off(i, j)]; }
    T& operator()(int i, int j, int k) { return first_[off(i, j, k)]; }
    const T& operator()(int i, int j, int k) const { return first_[off(i, j, k)]; }
    T& operator()(const TinyVector<int, N>& x) { return first_[offv(x.v)]; }
    const T& operator()(const TinyVector<int, N>& x) const { return first_[offv(x.v)]; }

    Array copy() const {
        Array r;
        r.allocate(ext_);
        for (int d = 0; d < N; ++d) r.base_[d] = base_[d];
        r.assign_from(*this);
        return r;
    }

    // --- assignment -------------------------------------------------------------------
    Array& operator=(const Array& o) {
        if (this == &o) return *this;
        if (!first_) {  // an empty array takes the other's shape
            allocate(o.ext_);
            for (int d = 0; d < N; ++d) base_[d] = o.base_[d];
        }
        assign_from(o);
        return *this;
    }
    Array& operator=(T s) {
        for_each_index([&](const int* x) { at(x) = s; });
        return *this;
    }
    Array& operator+=(T s) {
        for_each_index([&](const int* x) { at(x) += s; });
        return *this;
    }
    Array& operator-=(T s) {
        for_each_index([&](const int* x) { at(x) -= s; });
        return *this;
    }
    Array& operator*=(T s) {
        for_each_index([&](const int* x) { at(x) *= s; });
        return *this;
    }
    Array& operator/=(T s) {
        for_each_index([&](const int* x) { at(x) /= s; });
        return *this;
    }
    Array& operator+=(const Array& o) { return combine(o, [](T& a, T b) { a += b; }); }
    Array& operator-=(const Array& o) { return combine(o, [](T& a, T b) { a -= b; }); }
    Array& operator*=(const Array& o) { return combine(o, [](T& a, T b) { a *= b; }); }
    Array& operator/=(const Array& o) { return combine(o, [](T& a, T b) { a /= b; }); }

    // Walks the index domain in storage order; f receives the N indices.
    template <typename F>
    void for_each_index(F f) const {
        if (!first_) return;
        int x[N];
        for (int d = 0; d < N; ++d) {
            if (ext_[d] <= 0) return;
            x[d] = base_[d];
        }
        for (;;) {
            f(x);
            int d = N - 1;
            while (d >= 0) {
                if (++x[d] < base_[d] + ext_[d]) break;
                x[d] = base_[d];
                --d;
            }
            if (d < 0) return;
        }
    }
    T& at(const int* x) { return first_[offv(x)]; }
    const T& at(const int* x) const { return first_[offv(x)]; }

private:
    std::shared_ptr<T> store_;
    T* first_ = nullptr;  // element at the base index
    int base_[N] = {};
    int ext_[N] = {};
    ptrdiff_t stride_[N] = {};

    void init1(int e0) {
        int e[1] = {e0};
        allocate_n(e, 1);
    }
    void init2(int e0, int e1) {
        int e[2] = {e0, e1};
        allocate_n(e, 2);
    }
    void init3(int e0, int e1, int e2) {
        int e[3] = {e0, e1, e2};
        allocate_n(e, 3);
    }
    void allocate_n(const int* e, int n) {
        if (n != N) throw "blitz shim: wrong number of extents";
        allocate(e);
    }
    void allocate(const int* e) {
        size_t n = 1;
        for (int d = 0; d < N; ++d) {  // as in Blitz, resizing keeps the index base
            ext_[d] = e[d];
            n *= (size_t)(e[d] > 0 ? e[d] : 0);
        }
        ptrdiff_t s = 1;
        for (int d = N - 1; d >= 0; --d) {
            stride_[d] = s;
            s *= (ext_[d] > 0 ? ext_[d] : 0);
        }
        store_ = std::shared_ptr<T>(new T[n ? n : 1](), std::default_delete<T[]>());
        first_ = store_.get();
    }
    ptrdiff_t off(int i) const { return (ptrdiff_t)(i - base_[0]) * stride_[0]; }
    ptrdiff_t off(int i, int j) const {
        return (ptrdiff_t)(i - base_[0]) * stride_[0] + (ptrdiff_t)(j - base_[1]) * stride_[1];
    }
    ptrdiff_t off(int i, int j, int k) const {
        return (ptrdiff_t)(i - base_[0]) * stride_[0] + (ptrdiff_t)(j - base_[1]) * stride_[1] +
               (ptrdiff_t)(k - base_[2]) * stride_[2];
    }
    ptrdiff_t offv(const int* x) const {
        ptrdiff_t o = 0;
        for (int d = 0; d < N; ++d) o += (ptrdiff_t)(x[d] - base_[d]) * stride_[d];
        return o;
    }
    void assign_from(const Array& o) {
        // Elements are matched by index, as Blitz evaluates array expressions; a source that
        // views this array's own storage is copied first.
        Array src = o.copy_if_alias(*this);
        for_each_index([&](const int* x) { at(x) = src.at(x); });
    }
    Array copy_if_alias(const Array& dst) const {
        if (store_ && store_ == dst.store_) {
            Array r;
            r.allocate(ext_);
            for (int d = 0; d < N; ++d) r.base_[d] = base_[d];
            for_each_index([&](const int* x) { r.at(x) = at(x); });
            return r;
        }
        return *this;
    }
    template <typename Op>
    Array& combine(const Array& o, Op op) {
        Array src = o.copy_if_alias(*this);
        for_each_index([&](const int* x) { op(at(x), src.at(x)); });
        return *this;
    }
};

// Elementwise arithmetic: the result has the left operand's index base and extents.
#define IMPEC_BLITZ_SHIM_BINOP(OP)                                                     \
    template <typename T, int N>                                                       \
    Array<T, N> operator OP(const Array<T, N>& a, const Array<T, N>& b) {              \
        Array<T, N> r = a.copy();                                                      \
        r.for_each_index([&](const int* x) { r.at(x) = a.at(x) OP b.at(x); });         \
        return r;                                                                      \
    }                                                                                  \
    template <typename T, int N>                                                       \
    Array<T, N> operator OP(const Array<T, N>& a, T s) {                               \
        Array<T, N> r = a.copy();                                                      \
        r.for_each_index([&](const int* x) { r.at(x) = a.at(x) OP s; });              \
        return r;                                                                      \
    }                                                                                  \
    template <typename T, int N>                                                       \
    Array<T, N> operator OP(T s, const Array<T, N>& a) {                               \
        Array<T, N> r = a.copy();                                                      \
        r.for_each_index([&](const int* x) { r.at(x) = s OP a.at(x); });              \
        return r;                                                                      \
    }
IMPEC_BLITZ_SHIM_BINOP(+)
IMPEC_BLITZ_SHIM_BINOP(-)
IMPEC_BLITZ_SHIM_BINOP(*)
IMPEC_BLITZ_SHIM_BINOP(/)
#undef IMPEC_BLITZ_SHIM_BINOP

template <typename T, int N>
Array<T, N> operator-(const Array<T, N>& a) {
    Array<T, N> r = a.copy();
    r.for_each_index([&](const int* x) { r.at(x) = -a.at(x); });
    return r;
}

// Full reductions over every element (Blitz's max(expr), min(expr), sum(expr) of an array).
template <typename T, int N>
T max(const Array<T, N>& a) {
    T m = -std::numeric_limits<T>::max();
    a.for_each_index([&](const int* x) {
        if (a.at(x) > m) m = a.at(x);
    });
    return m;
}
template <typename T, int N>
T min(const Array<T, N>& a) {
    T m = std::numeric_limits<T>::max();
    a.for_each_index([&](const int* x) {
        if (a.at(x) < m) m = a.at(x);
    });
    return m;
}
template <typename T, int N>
T sum(const Array<T, N>& a) {
    T m = T();
    a.for_each_index([&](const int* x) { m += a.at(x); });
    return m;
}

template <typename T, int N>
std::ostream& operator<<(std::ostream& os, const TinyVector<T, N>& t) {
    os << "(";
    for (int d = 0; d < N; ++d) os << (d ? "," : "") << t[d];
    return os << ")";
}

}  // namespace blitz

#endif
