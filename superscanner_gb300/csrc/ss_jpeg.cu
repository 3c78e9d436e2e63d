// ss_jpeg.cu — colour frames of a recording (src/cameras/DataCam.cpp:30-46,
// 66-69: color/<NNNNNN>.jpg first, .png as the fallback, resized to the frame
// size with cv::resize's default interpolation). A JPEG is decoded on the GPU
// by nvJPEG (the CUDA toolkit's JPEG library, loaded at run time so that
// libss.so does not depend on it: only these entry points fail without it)
// into interleaved RGB in device memory, then resized by bilinear sampling
// with cv::resize's INTER_LINEAR geometry: the source coordinate of
// destination pixel d is (d + 0.5) src / dst - 0.5, clamped to the first and
// last pixel. OpenCV weighs the four pixels with 11-bit fixed-point
// coefficients; here they are FP32, so a value can differ by one.
#include <dlfcn.h>
#include <nvjpeg.h>

#include "ss_grid_impl.cuh"

struct ss_jpeg {
    void *lib = nullptr;
    decltype(&nvjpegCreateSimple) create = nullptr;
    decltype(&nvjpegDestroy) destroy = nullptr;
    decltype(&nvjpegJpegStateCreate) state_create = nullptr;
    decltype(&nvjpegJpegStateDestroy) state_destroy = nullptr;
    decltype(&nvjpegGetImageInfo) info = nullptr;
    decltype(&nvjpegDecode) decode = nullptr;
    nvjpegHandle_t h = nullptr;
    nvjpegJpegState_t st = nullptr;
    unsigned char *tmp = nullptr;  // decoded image before resizing (device)
    size_t tmp_bytes = 0;
};

namespace ss {

// Bilinear resize of interleaved 8-bit RGB (cv::resize INTER_LINEAR geometry).
__global__ void resize_rgb_kernel(const unsigned char *__restrict__ src, int sh, int sw,
                                  unsigned char *__restrict__ dst, int dh, int dw) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= dh || j >= dw) return;
    const float fy = ((float)i + 0.5f) * ((float)sh / (float)dh) - 0.5f;
    const float fx = ((float)j + 0.5f) * ((float)sw / (float)dw) - 0.5f;
    int y0 = (int)floorf(fy), x0 = (int)floorf(fx);
    float ay = fy - (float)y0, ax = fx - (float)x0;
    if (y0 < 0) y0 = 0, ay = 0.f;
    if (x0 < 0) x0 = 0, ax = 0.f;
    if (y0 >= sh - 1) y0 = sh - 1, ay = 0.f;
    if (x0 >= sw - 1) x0 = sw - 1, ax = 0.f;
    const int y1 = min(y0 + 1, sh - 1), x1 = min(x0 + 1, sw - 1);
    const unsigned char *p00 = src + ((size_t)y0 * sw + x0) * 3, *p01 = src + ((size_t)y0 * sw + x1) * 3;
    const unsigned char *p10 = src + ((size_t)y1 * sw + x0) * 3, *p11 = src + ((size_t)y1 * sw + x1) * 3;
    unsigned char *q = dst + ((size_t)i * dw + j) * 3;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const float top = fmaf(ax, (float)p01[c] - (float)p00[c], (float)p00[c]);
        const float bot = fmaf(ax, (float)p11[c] - (float)p10[c], (float)p10[c]);
        const float v = fmaf(ay, bot - top, top);
        q[c] = (unsigned char)fminf(fmaxf(rintf(v), 0.f), 255.f);
    }
}

}  // namespace ss

using namespace ss;

namespace {

template <class F>
bool load_sym(void *lib, const char *name, F &f) {
    f = reinterpret_cast<F>(dlsym(lib, name));
    return f != nullptr;
}

ss_status nvjpeg_status(const char *where, nvjpegStatus_t e) {
    if (e == NVJPEG_STATUS_SUCCESS) return SS_OK;
    set_last_error_text(std::string(where) + ": nvJPEG status " + std::to_string((int)e));
    return e == NVJPEG_STATUS_BAD_JPEG || e == NVJPEG_STATUS_JPEG_NOT_SUPPORTED || e == NVJPEG_STATUS_INVALID_PARAMETER
               ? SS_ERR_ARG
               : SS_ERR_CUDA;
}

}  // namespace

extern "C" {

ss_status ss_jpeg_create(ss_jpeg **out) {
    if (!out) return SS_ERR_ARG;
    *out = nullptr;
    void *lib = dlopen("libnvjpeg.so.13", RTLD_NOW | RTLD_LOCAL);
    if (!lib) lib = dlopen("libnvjpeg.so", RTLD_NOW | RTLD_LOCAL);
    if (!lib) {
        set_last_error_text("ss_jpeg_create: libnvjpeg (CUDA toolkit) not found");
        return SS_ERR_STATE;
    }
    ss_jpeg *j = new ss_jpeg;
    j->lib = lib;
    const bool ok = load_sym(lib, "nvjpegCreateSimple", j->create) && load_sym(lib, "nvjpegDestroy", j->destroy) &&
                    load_sym(lib, "nvjpegJpegStateCreate", j->state_create) &&
                    load_sym(lib, "nvjpegJpegStateDestroy", j->state_destroy) &&
                    load_sym(lib, "nvjpegGetImageInfo", j->info) && load_sym(lib, "nvjpegDecode", j->decode);
    if (!ok) {
        set_last_error_text("ss_jpeg_create: libnvjpeg lacks an entry point");
        dlclose(lib);
        delete j;
        return SS_ERR_STATE;
    }
    ss_status st = nvjpeg_status("nvjpegCreateSimple", j->create(&j->h));
    if (st == SS_OK) st = nvjpeg_status("nvjpegJpegStateCreate", j->state_create(j->h, &j->st));
    if (st != SS_OK) {
        ss_jpeg_destroy(j);
        return st;
    }
    *out = j;
    return SS_OK;
}

ss_status ss_jpeg_destroy(ss_jpeg *j) {
    if (!j) return SS_ERR_ARG;
    if (j->st) j->state_destroy(j->st);
    if (j->h) j->destroy(j->h);
    cudaFree(j->tmp);
    if (j->lib) dlclose(j->lib);
    delete j;
    return SS_OK;
}

ss_status ss_jpeg_info(ss_jpeg *j, const uint8_t *data, size_t size, int32_t *rows, int32_t *cols) {
    if (!j || !data || !size || !rows || !cols) return SS_ERR_ARG;
    int nc = 0, w[NVJPEG_MAX_COMPONENT] = {}, h[NVJPEG_MAX_COMPONENT] = {};
    nvjpegChromaSubsampling_t sub;
    ss_status st = nvjpeg_status("nvjpegGetImageInfo", j->info(j->h, data, size, &nc, &sub, w, h));
    if (st != SS_OK) return st;
    if (nc != 1 && nc != 3) return SS_ERR_ARG;
    *rows = h[0];
    *cols = w[0];
    return SS_OK;
}

ss_status ss_jpeg_decode_rgb(ss_jpeg *j, const uint8_t *data, size_t size, uint8_t *rgb, int32_t rows, int32_t cols,
                             ss_stream_t stream) {
    if (!j || !data || !size || !rgb || rows <= 0 || cols <= 0) return SS_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    int32_t h = 0, w = 0;
    ss_status st = ss_jpeg_info(j, data, size, &h, &w);
    if (st != SS_OK) return st;
    const bool same = h == rows && w == cols;
    unsigned char *out = rgb;
    if (!same) {
        const size_t bytes = (size_t)h * w * 3;
        if (bytes > j->tmp_bytes) {
            cudaFree(j->tmp);
            j->tmp = nullptr;
            j->tmp_bytes = 0;
            SS_CUDA_TRY(cudaMalloc(&j->tmp, bytes));
            j->tmp_bytes = bytes;
        }
        out = j->tmp;
    }
    nvjpegImage_t img = {};
    img.channel[0] = out;
    img.pitch[0] = (size_t)w * 3;
    st = nvjpeg_status("nvjpegDecode", j->decode(j->h, j->st, data, size, NVJPEG_OUTPUT_RGBI, &img, s));
    if (st != SS_OK) return st;
    if (!same) {
        const dim3 blk(32, 8), grid((cols + 31) / 32, (rows + 7) / 8);
        resize_rgb_kernel<<<grid, blk, 0, s>>>(j->tmp, h, w, rgb, rows, cols);
        SS_LAUNCH_CHECK();
    }
    return SS_OK;
}

ss_status ss_resize_rgb(const uint8_t *src, int32_t src_rows, int32_t src_cols, uint8_t *dst, int32_t rows,
                        int32_t cols, ss_stream_t stream) {
    if (!src || !dst || src_rows <= 0 || src_cols <= 0 || rows <= 0 || cols <= 0) return SS_ERR_ARG;
    const dim3 blk(32, 8), grid((cols + 31) / 32, (rows + 7) / 8);
    resize_rgb_kernel<<<grid, blk, 0, (cudaStream_t)stream>>>(src, src_rows, src_cols, dst, rows, cols);
    SS_LAUNCH_CHECK();
    return SS_OK;
}

}  // extern "C"
