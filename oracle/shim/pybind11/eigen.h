// numpy (2-D, any numeric dtype) <-> Eigen-stand-in complex row-major matrix
// caster, shadowing pybind11/eigen.h for the reference CPU module build (test
// infrastructure).  Used by instructions.hpp:252-261 (.cast<RowMatrixXcd>()).
#pragma once
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>

#include <Eigen/Core>
#include <complex>

namespace pybind11 {
namespace detail {
template <>
struct type_caster<Eigen::Matrix<std::complex<double>, Eigen::Dynamic, Eigen::Dynamic, Eigen::RowMajor>> {
    using Mat = Eigen::Matrix<std::complex<double>, Eigen::Dynamic, Eigen::Dynamic, Eigen::RowMajor>;
    PYBIND11_TYPE_CASTER(Mat, const_name("numpy.ndarray[complex128[m, n]]"));

    bool load(handle src, bool) {
        auto arr = array_t<std::complex<double>, array::c_style | array::forcecast>::ensure(src);
        if (!arr) return false;
        if (arr.ndim() == 1) {
            value = Mat(arr.shape(0), 1);
        } else if (arr.ndim() == 2) {
            value = Mat(arr.shape(0), arr.shape(1));
        } else {
            return false;
        }
        const std::complex<double>* p = arr.data();
        for (long i = 0; i < value.size(); ++i) value.data()[i] = p[i];
        return true;
    }

    static handle cast(const Mat& m, return_value_policy, handle) {
        array_t<std::complex<double>> a({m.rows(), m.cols()});
        auto* p = a.mutable_data();
        for (long i = 0; i < m.size(); ++i) p[i] = m.data()[i];
        return a.release();
    }
};
}  // namespace detail
}  // namespace pybind11
