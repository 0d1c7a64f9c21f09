// ref_shim.cuh -- TEST INFRASTRUCTURE.  Stand-ins for the parts of the
// reference's absent dependencies (imageutilities' iu:: containers and
// helper math, the ndarray_ref view) that the reference's own CUDA kernels
// use, so that those kernels compile unchanged into a device-code module
// that the tests run as a second oracle (oracle/build_ref.py,
// oracle/ref_host.cpp).  Nothing here is product code.
//
// Each type is restated from how the reference's kernels and launchers use
// it (the library's sources are not in the reference tree):
//  - ImageGpu_*::KernelData: a pitched image (iu::ImageGpu, allocated with
//    cudaMallocPitch); data_[y * stride_ + x], stride_ in elements
//    (stereo/stereo.cu:711, 816: `y*u.stride_+x`), width_, height_.
//  - LinearDeviceMemory_32f_C1::KernelData: a flat array; d(i) = data_[i]
//    (stereo/operators/stereocorrelation.cu:46, stereo/stereo.cu:330).
//  - TensorGpu_32f::TensorKernelData: a 4-D tensor in NCHW or NHWC memory
//    order; t(a, b, c, d) and coords() index in memory order -- im0(n, c, h, w)
//    on NCHW features, out(n, h, w, d) on the NHWC volume
//    (stereo/operators/stereocorrelation.cu:41-58), volume(0, y, x, k) on the
//    3-label NHWC volume (stereo/stereo.cu:424); C, H, W are the tensor's
//    channel, height and width, length_ its element count.
//  - kernel::ndarray_ref<float, 3>: a strided 3-D view; size(i), v(i, j, k)
//    (stereo/stereo.cu:917-924 on get_C1().permute_dims({1, 2, 0}),
//    stereo/stereo.cpp:408).
//  - helper math: make_float2(s), float2 arithmetic with floats and float2s,
//    clamp(v, lo, hi) = max(lo, min(v, hi)) for float and float2 (the
//    argument order of stereo/stereo.cu:723,756,792).
#ifndef CNNCRF_REF_SHIM_CUH
#define CNNCRF_REF_SHIM_CUH

#include <cuda_runtime.h>
#include <cfloat>

#include <cmath>

namespace iu {

template <class T> struct PitchedKernelData {
    T *data_;
    int width_, height_, stride_;
    __host__ __device__ T &operator()(int x, int y) { return data_[y * stride_ + x]; }
    __host__ __device__ const T &operator()(int x, int y) const { return data_[y * stride_ + x]; }
};

struct ImageGpu_32f_C1 { using KernelData = PitchedKernelData<float>; };
struct ImageGpu_32f_C2 { using KernelData = PitchedKernelData<float2>; };
struct ImageGpu_32f_C4 { using KernelData = PitchedKernelData<float4>; };
struct ImageGpu_32s_C1 { using KernelData = PitchedKernelData<int>; };

struct LinearDeviceMemory_32f_C1 {
    struct KernelData {
        float *data_;
        int length_;
        __host__ __device__ float &operator()(int i) { return data_[i]; }
    };
};

struct TensorGpu_32f {
    struct TensorKernelData {
        float *data_;
        unsigned int length_;
        int N, C, H, W;
        int nhwc; // memory order: 0 NCHW, 1 NHWC
        // extents in memory order
        __host__ __device__ int d1() const { return nhwc ? H : C; }
        __host__ __device__ int d2() const { return nhwc ? W : H; }
        __host__ __device__ int d3() const { return nhwc ? C : W; }
        __host__ __device__ float &operator()(int a, int b, int c, int d)
        {
            return data_[((long)(a * d1() + b) * d2() + c) * d3() + d];
        }
        __host__ __device__ void coords(unsigned int idx, short *a, short *b, short *c, short *d) const
        {
            *d = (short)(idx % d3());
            idx /= d3();
            *c = (short)(idx % d2());
            idx /= d2();
            *b = (short)(idx % d1());
            *a = (short)(idx / d1());
        }
    };
};

} // namespace iu

namespace kernel {
template <class T, int N> struct ndarray_ref {
    T *data_;
    int size_[N];
    long stride_[N]; // in elements
    __host__ __device__ int size(int i) const { return size_[i]; }
    __host__ __device__ T &operator()(int i, int j, int k) const
    {
        return data_[i * stride_[0] + j * stride_[1] + k * stride_[2]];
    }
};
} // namespace kernel

// helper math
inline __host__ __device__ float2 make_float2(float s) { return make_float2(s, s); }
inline __host__ __device__ float2 operator+(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
inline __host__ __device__ float2 operator-(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
inline __host__ __device__ float2 operator-(float2 a) { return make_float2(-a.x, -a.y); }
inline __host__ __device__ float2 operator*(float s, float2 a) { return make_float2(s * a.x, s * a.y); }
inline __host__ __device__ float2 operator*(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
inline __host__ __device__ float2 operator/(float2 a, float s) { return make_float2(a.x / s, a.y / s); }
inline __device__ float clamp(float v, float lo, float hi) { return fmaxf(lo, fminf(v, hi)); }
inline __device__ float2 clamp(float2 v, float2 lo, float2 hi)
{
    return make_float2(clamp(v.x, lo.x, hi.x), clamp(v.y, lo.y, hi.y));
}

#endif
