// Ghost-indexed host arrays with the subset of the Blitz++ Array2d / Array3d interface that the
// reference's class surface uses (src/GenSimDefs.h:22-31): base indices may be negative
// (ghost cells), the last index is contiguous (row-major), k is innermost for Array3d.
#pragma once
#include <algorithm>
#include <cstddef>
#include <vector>

class Array2d {
public:
    Array2d() = default;
    Array2d(int n0, int n1, int b0 = 0, int b1 = 0) { resize(n0, n1, b0, b1); }
    void resize(int n0, int n1, int b0 = 0, int b1 = 0) {
        n0_ = n0; n1_ = n1; b0_ = b0; b1_ = b1;
        d_.assign((size_t)n0 * n1, 0.0);
    }
    double& operator()(int i, int j) { return d_[(size_t)(i - b0_) * n1_ + (j - b1_)]; }
    double operator()(int i, int j) const { return d_[(size_t)(i - b0_) * n1_ + (j - b1_)]; }
    int base(int r) const { return r == 0 ? b0_ : b1_; }
    int extent(int r) const { return r == 0 ? n0_ : n1_; }
    double* data() { return d_.data(); }
    const double* data() const { return d_.data(); }
    size_t size() const { return d_.size(); }
    Array2d& operator=(double v) { std::fill(d_.begin(), d_.end(), v); return *this; }
    double max() const { return *std::max_element(d_.begin(), d_.end()); }
    double min() const { return *std::min_element(d_.begin(), d_.end()); }

private:
    int n0_ = 0, n1_ = 0, b0_ = 0, b1_ = 0;
    std::vector<double> d_;
};

class Array3d {
public:
    Array3d() = default;
    void resize(int n0, int n1, int n2, int b0 = 0, int b1 = 0) {
        n0_ = n0; n1_ = n1; n2_ = n2; b0_ = b0; b1_ = b1;
        d_.assign((size_t)n0 * n1 * n2, 0.0);
    }
    double& operator()(int i, int j, int k) { return d_[((size_t)(i - b0_) * n1_ + (j - b1_)) * n2_ + k]; }
    double operator()(int i, int j, int k) const { return d_[((size_t)(i - b0_) * n1_ + (j - b1_)) * n2_ + k]; }
    int base(int r) const { return r == 0 ? b0_ : (r == 1 ? b1_ : 0); }
    int extent(int r) const { return r == 0 ? n0_ : (r == 1 ? n1_ : n2_); }
    double* data() { return d_.data(); }
    const double* data() const { return d_.data(); }
    Array3d& operator=(double v) { std::fill(d_.begin(), d_.end(), v); return *this; }

private:
    int n0_ = 0, n1_ = 0, n2_ = 2, b0_ = 0, b1_ = 0;
    std::vector<double> d_;
};
