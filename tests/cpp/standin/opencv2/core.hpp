// Stand-in for the members of cv::Mat and cv::cuda::GpuMat that
// include/yas_rgbdfusion.hpp (with YAS_SHIM_OPENCV) and FullSystem's
// Tracking.cpp use: 2-D images of CV_8UC1 / CV_32FC1 / CV_32FC4 with row
// pitch, reference-counted storage, host<->device copies (GpuMat::upload,
// download, and the cv::Mat(GpuMat) download constructor) through the CUDA
// runtime.  Test infrastructure only: it lets the shim's OpenCV branch compile
// and run where OpenCV is absent.
#pragma once

#include <cuda_runtime_api.h>

#include <cstddef>
#include <cstring>
#include <memory>
#include <stdexcept>

#define CV_8U 0
#define CV_32F 5
#define CV_8UC1 0
#define CV_32FC1 5
#define CV_32FC4 29

namespace cv {

inline size_t elem_size_of(int type) {
    const int depth = type & 7, cn = (type >> 3) + 1;
    return (size_t)(depth == CV_32F ? 4 : 1) * (size_t)cn;
}

namespace cuda {
class GpuMat;
}

class Mat {
public:
    Mat() = default;
    Mat(int rows_, int cols_, int type_) : rows(rows_), cols(cols_), step((size_t)cols_ * elem_size_of(type_)), type_(type_) {
        auto buf = std::shared_ptr<unsigned char>(new unsigned char[step * (size_t)rows_ + 1](),
                                                  std::default_delete<unsigned char[]>());
        data = buf.get();
        owner_ = buf;
    }
    Mat(int rows_, int cols_, int type_, void *data_, size_t step_ = 0)
        : data(static_cast<unsigned char *>(data_)), rows(rows_), cols(cols_),
          step(step_ ? step_ : (size_t)cols_ * elem_size_of(type_)), type_(type_) {}
    explicit Mat(const cuda::GpuMat &m);  // downloads, as cv::Mat(const cuda::GpuMat&)

    size_t elemSize() const { return elem_size_of(type_); }
    int type() const { return type_; }
    bool empty() const { return data == nullptr || rows == 0 || cols == 0; }
    template <typename T>
    T *ptr(int r = 0) {
        return reinterpret_cast<T *>(data + (size_t)r * step);
    }
    template <typename T>
    const T *ptr(int r = 0) const {
        return reinterpret_cast<const T *>(data + (size_t)r * step);
    }

    unsigned char *data = nullptr;
    int rows = 0, cols = 0;
    size_t step = 0;

private:
    int type_ = 0;
    std::shared_ptr<unsigned char> owner_;
};

namespace cuda {

class GpuMat {
public:
    GpuMat() = default;
    GpuMat(int rows_, int cols_, int type_) { create(rows_, cols_, type_); }
    GpuMat(int rows_, int cols_, int type_, void *data_, size_t step_)
        : data(static_cast<unsigned char *>(data_)), rows(rows_), cols(cols_), step(step_), type_(type_) {}

    void create(int rows_, int cols_, int type_x) {
        if (rows == rows_ && cols == cols_ && type_ == type_x && owner_) return;
        void *p = nullptr;
        size_t pitch = 0;
        if (cudaMallocPitch(&p, &pitch, (size_t)cols_ * elem_size_of(type_x), (size_t)rows_) != cudaSuccess)
            throw std::runtime_error("GpuMat::create: cudaMallocPitch failed");
        owner_ = std::shared_ptr<unsigned char>(static_cast<unsigned char *>(p), [](unsigned char *q) { cudaFree(q); });
        data = owner_.get();
        rows = rows_, cols = cols_, step = pitch, type_ = type_x;
    }
    void upload(const Mat &m) {
        create(m.rows, m.cols, m.type());
        if (cudaMemcpy2D(data, step, m.data, m.step, (size_t)cols * elemSize(), (size_t)rows, cudaMemcpyHostToDevice) !=
            cudaSuccess)
            throw std::runtime_error("GpuMat::upload failed");
    }
    void download(Mat &m) const {
        if (m.rows != rows || m.cols != cols || m.type() != type_ || m.empty()) m = Mat(rows, cols, type_);
        if (cudaMemcpy2D(m.data, m.step, data, step, (size_t)cols * elemSize(), (size_t)rows, cudaMemcpyDeviceToHost) !=
            cudaSuccess)
            throw std::runtime_error("GpuMat::download failed");
    }
    size_t elemSize() const { return elem_size_of(type_); }
    int type() const { return type_; }
    bool empty() const { return data == nullptr || rows == 0 || cols == 0; }
    template <typename T>
    T *ptr(int r = 0) {
        return reinterpret_cast<T *>(data + (size_t)r * step);
    }

    unsigned char *data = nullptr;
    int rows = 0, cols = 0;
    size_t step = 0;

private:
    int type_ = 0;
    std::shared_ptr<unsigned char> owner_;
};

}  // namespace cuda

inline Mat::Mat(const cuda::GpuMat &m) { m.download(*this); }

}  // namespace cv
