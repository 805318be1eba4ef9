// Stand-in for the members of Sophus::SE3d that include/yas_rgbdfusion.hpp
// (with YAS_SHIM_SOPHUS) and FullSystem's Tracking.cpp call: construction from
// a 4x4 matrix or (R, t), matrix(), matrix3x4(), translation(), inverse() and
// composition.  Test infrastructure only: rotation kept as a 3x3 matrix (the
// real class keeps a unit quaternion).
#pragma once

#include <Eigen/Core>

namespace Sophus {

class SE3d {
public:
    SE3d() : R_(Eigen::Matrix3d::Identity()), t_() {}
    explicit SE3d(const Eigen::Matrix4d &T) {
        for (int r = 0; r < 3; ++r) {
            for (int c = 0; c < 3; ++c) R_(r, c) = T(r, c);
            t_(r) = T(r, 3);
        }
    }
    SE3d(const Eigen::Matrix3d &R, const Eigen::Vector3d &t) : R_(R), t_(t) {}

    Eigen::Matrix4d matrix() const {
        Eigen::Matrix4d M = Eigen::Matrix4d::Identity();
        for (int r = 0; r < 3; ++r) {
            for (int c = 0; c < 3; ++c) M(r, c) = R_(r, c);
            M(r, 3) = t_(r);
        }
        return M;
    }
    Eigen::Matrix<double, 3, 4> matrix3x4() const {
        Eigen::Matrix<double, 3, 4> M;
        for (int r = 0; r < 3; ++r) {
            for (int c = 0; c < 3; ++c) M(r, c) = R_(r, c);
            M(r, 3) = t_(r);
        }
        return M;
    }
    const Eigen::Vector3d &translation() const { return t_; }
    const Eigen::Matrix3d &rotationMatrix() const { return R_; }

    // [R | t]^-1 = [R^T | -R^T t], sums in the index order below
    SE3d inverse() const {
        SE3d o;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) o.R_(i, j) = R_(j, i);
        for (int i = 0; i < 3; ++i) o.t_(i) = -(o.R_(i, 0) * t_(0) + o.R_(i, 1) * t_(1) + o.R_(i, 2) * t_(2));
        return o;
    }
    // [Ra | ta] [Rb | tb] = [Ra Rb | Ra tb + ta]
    SE3d operator*(const SE3d &b) const {
        SE3d o;
        for (int i = 0; i < 3; ++i) {
            for (int j = 0; j < 3; ++j) o.R_(i, j) = R_(i, 0) * b.R_(0, j) + R_(i, 1) * b.R_(1, j) + R_(i, 2) * b.R_(2, j);
            o.t_(i) = R_(i, 0) * b.t_(0) + R_(i, 1) * b.t_(1) + R_(i, 2) * b.t_(2) + t_(i);
        }
        return o;
    }

private:
    Eigen::Matrix3d R_;
    Eigen::Vector3d t_;
};

}  // namespace Sophus
