// Stand-in: cv::cuda::GpuMat lives in opencv2/core.hpp of this stand-in.
#pragma once

#include <opencv2/core.hpp>
