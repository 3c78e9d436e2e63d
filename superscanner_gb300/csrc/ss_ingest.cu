// ss_ingest.cu — host-side help for reading the reference's frame files
// (src/cameras/DataCam.cpp:10-100: depth/<NNNNNN>.png, 16-bit grey; colour
// PNGs): the PNG row filters undone (the sequential Sub, Average and Paeth
// filters are too slow to run per byte from Python). Host code only.
#include <cstdint>
#include <cstdlib>

#include "ss_grid_impl.cuh"

extern "C" ss_status ss_png_unfilter(const uint8_t *filtered, int32_t rows, int32_t row_bytes, int32_t bpp,
                                     uint8_t *out) {
    // PNG filter types 0..4 (None, Sub, Up, Average, Paeth); each filtered row
    // is one filter-type byte followed by row_bytes bytes.
    if (!filtered || !out || rows < 0 || row_bytes < 0 || bpp < 1 || bpp > 8) return SS_ERR_ARG;
    for (int32_t r = 0; r < rows; r++) {
        const uint8_t type = filtered[(size_t)r * (row_bytes + 1)];
        const uint8_t *src = filtered + (size_t)r * (row_bytes + 1) + 1;
        uint8_t *dst = out + (size_t)r * row_bytes;
        const uint8_t *up = r > 0 ? out + (size_t)(r - 1) * row_bytes : nullptr;
        for (int32_t k = 0; k < row_bytes; k++) {
            const int a = k >= bpp ? dst[k - bpp] : 0, b = up ? up[k] : 0, c = (up && k >= bpp) ? up[k - bpp] : 0;
            int pred;
            switch (type) {
                case 0: pred = 0; break;
                case 1: pred = a; break;
                case 2: pred = b; break;
                case 3: pred = (a + b) >> 1; break;
                case 4: {
                    const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
                    pred = (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
                    break;
                }
                default: return SS_ERR_ARG;
            }
            dst[k] = (uint8_t)(src[k] + pred);
        }
    }
    return SS_OK;
}
