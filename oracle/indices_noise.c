/*
 * indices_noise.c — oracle of the index buffer and the noise heightmap.
 * Test infrastructure only (see wt_oracle.h); never used by the product.
 */
#include <math.h>
#include <stdlib.h>
#include "wt_oracle.h"

/* src/program.cpp:686-717: gridIndices[row][col] = row*L + col (:694-699),
 * then per cell (row, col) of the (L-1)^2 cells, in row-major order,
 * (r,c) (r+1,c+1) (r+1,c) and (r,c) (r,c+1) (r+1,c+1) (:703-716).
 * Generalised to cols x rows and a base vertex (0 and 513 x 513 there). */
void wto_grid_indices(uint32_t cols, uint32_t rows, uint32_t base_vertex, uint32_t* out) {
    size_t k = 0;
    for (uint32_t row = 0; row + 1 < rows; ++row) {
        for (uint32_t col = 0; col + 1 < cols; ++col) {
            uint32_t i00 = base_vertex + row * cols + col;
            uint32_t i01 = base_vertex + row * cols + col + 1;
            uint32_t i10 = base_vertex + (row + 1) * cols + col;
            uint32_t i11 = base_vertex + (row + 1) * cols + col + 1;
            out[k++] = i00; out[k++] = i11; out[k++] = i10;
            out[k++] = i00; out[k++] = i01; out[k++] = i11;
        }
    }
}

/* h(i, j) = sum_m a_m sin(2*pi*(kx_m*i/width + ky_m*j/height) + psi_m + r_m*t),
 * then (h - min) / (max - min).  Integer wavenumbers make it tile; rates
 * (NULL = none) animate it in time. */
void wto_noise_f64_at(const wt_noise_term* terms, uint32_t n_terms, const float* rates, double time_s,
                      uint32_t width, uint32_t height, double* out) {
    const double two_pi = 6.283185307179586476925286766559;
    double lo = INFINITY, hi = -INFINITY;
    for (uint32_t j = 0; j < height; ++j)
        for (uint32_t i = 0; i < width; ++i) {
            double h = 0.0;
            for (uint32_t m = 0; m < n_terms; ++m) {
                /* reduce the integer products exactly before scaling */
                long long ni = ((long long)terms[m].kx * i) % (long long)width;
                long long nj = ((long long)terms[m].ky * j) % (long long)height;
                double turns = (double)ni / width + (double)nj / height;
                double psi = (double)terms[m].phase + (rates ? (double)rates[m] * time_s : 0.0);
                h += (double)terms[m].amplitude * sin(two_pi * turns + psi);
            }
            out[(size_t)j * width + i] = h;
            if (h < lo) lo = h;
            if (h > hi) hi = h;
        }
    double span = hi - lo;
    size_t n = (size_t)width * height;
    for (size_t v = 0; v < n; ++v) out[v] = span > 0.0 ? (out[v] - lo) / span : 0.0;
}

void wto_noise_f64(const wt_noise_term* terms, uint32_t n_terms, uint32_t width,
                   uint32_t height, double* out) {
    wto_noise_f64_at(terms, n_terms, NULL, 0.0, width, height, out);
}
