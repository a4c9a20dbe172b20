// gen.cpp -- seeded synthetic CSR matrices (include/spmv_gen.h).  Host code only.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/spmv_gen.h"

namespace {

inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
// counter-based stream: draw k of stream (seed, idx)
inline uint64_t draw(uint64_t seed, uint64_t idx, uint64_t k = 0) {
    return mix64(mix64(seed ^ 0x5851F42D4C957F2Dull) ^ mix64(idx * 0x2545F4914F6CDD1Dull + k));
}
inline double unit(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
inline double unit_open0(uint64_t h) { return ((double)(h >> 11) + 1.0) * (1.0 / 9007199254740992.0); }  // (0,1]

// Poisson(lambda) by inversion over a counter stream (lambda up to a few hundred)
int poisson(double lambda, uint64_t seed, uint64_t idx) {
    if (lambda <= 0) return 0;
    if (lambda > 500) {  // normal approximation for large means
        double u1 = unit_open0(draw(seed, idx, 1)), u2 = unit(draw(seed, idx, 2));
        double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
        double v = std::floor(lambda + std::sqrt(lambda) * z + 0.5);
        return v < 0 ? 0 : (int)v;
    }
    double u = unit(draw(seed, idx, 3));
    double p = std::exp(-lambda), cdf = p;
    int k = 0;
    while (u > cdf && k < 100000) {
        ++k;
        p *= lambda / k;
        cdf += p;
    }
    return k;
}

int64_t finish_rows(int m, const std::vector<int64_t>& len, int* row_ptr) {
    int64_t acc = 0;
    row_ptr[0] = 0;
    for (int i = 0; i < m; ++i) {
        acc += len[i];
        if (acc > INT_MAX) return -1;
        row_ptr[i + 1] = (int)acc;
    }
    return acc;
}

}  // namespace

extern "C" int bhsp_gen_uniform(int64_t count, uint64_t seed, double lo, double hi, double* out) {
    if (count < 0 || (count > 0 && !out)) return -1;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < count; ++i) out[i] = lo + (hi - lo) * unit(draw(seed, (uint64_t)i));
    return 0;
}

extern "C" int bhsp_gen_uniform_int(int64_t count, uint64_t seed, int modulus, double* out) {
    if (count < 0 || modulus < 1 || (count > 0 && !out)) return -1;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < count; ++i) out[i] = (double)(draw(seed, (uint64_t)i) % (uint64_t)modulus);
    return 0;
}

extern "C" int64_t bhsp_gen_stencil2d_nnz(int nx, int ny) {
    if (nx < 1 || ny < 1) return -1;
    return (int64_t)nx * ny + 2ll * (nx - 1) * ny + 2ll * nx * (ny - 1);
}

extern "C" int bhsp_gen_stencil2d(int nx, int ny, double noise, uint64_t seed, int* row_ptr,
                                  int* col, double* val) {
    const int64_t nnz = bhsp_gen_stencil2d_nnz(nx, ny);
    if (nnz < 0 || nnz > INT_MAX || (int64_t)nx * ny > INT_MAX) return -1;
    const int m = nx * ny;
    row_ptr[0] = 0;
    for (int r = 0; r < m; ++r) {
        const int i = r / ny, j = r % ny;
        row_ptr[r + 1] = row_ptr[r] + 1 + (i > 0) + (i < nx - 1) + (j > 0) + (j < ny - 1);
    }
#pragma omp parallel for schedule(static)
    for (int r = 0; r < m; ++r) {
        const int i = r / ny, j = r % ny;
        int e = row_ptr[r];
        auto put = [&](int c, double w) {
            col[e] = c;
            val[e] = w + noise * (2.0 * unit(draw(seed, (uint64_t)e)) - 1.0);
            ++e;
        };
        if (i > 0) put(r - ny, -1.0);
        if (j > 0) put(r - 1, -1.0);
        put(r, 4.0);
        if (j < ny - 1) put(r + 1, -1.0);
        if (i < nx - 1) put(r + ny, -1.0);
    }
    return 0;
}

extern "C" int64_t bhsp_gen_stencil3d_nnz(int nx, int ny, int nz) {
    if (nx < 1 || ny < 1 || nz < 1) return -1;
    return (int64_t)(3 * (int64_t)nx - 2) * (3 * (int64_t)ny - 2) * (3 * (int64_t)nz - 2);
}

extern "C" int bhsp_gen_stencil3d(int nx, int ny, int nz, double noise, uint64_t seed,
                                  int* row_ptr, int* col, double* val) {
    const int64_t nnz = bhsp_gen_stencil3d_nnz(nx, ny, nz);
    const int64_t m64 = (int64_t)nx * ny * nz;
    if (nnz < 0 || nnz > INT_MAX || m64 > INT_MAX) return -1;
    const int m = (int)m64;
    auto cnt = [](int a, int n) { return 1 + (a > 0) + (a < n - 1); };
    row_ptr[0] = 0;
    for (int r = 0; r < m; ++r) {
        const int k = r % nz, j = (r / nz) % ny, i = r / (nz * ny);
        row_ptr[r + 1] = row_ptr[r] + cnt(i, nx) * cnt(j, ny) * cnt(k, nz);
    }
#pragma omp parallel for schedule(static)
    for (int r = 0; r < m; ++r) {
        const int k = r % nz, j = (r / nz) % ny, i = r / (nz * ny);
        int e = row_ptr[r];
        for (int di = -1; di <= 1; ++di) {
            if (i + di < 0 || i + di >= nx) continue;
            for (int dj = -1; dj <= 1; ++dj) {
                if (j + dj < 0 || j + dj >= ny) continue;
                for (int dk = -1; dk <= 1; ++dk) {
                    if (k + dk < 0 || k + dk >= nz) continue;
                    const int c = ((i + di) * ny + (j + dj)) * nz + (k + dk);
                    const double w = (di == 0 && dj == 0 && dk == 0) ? 26.0 : -1.0;
                    col[e] = c;
                    val[e] = w * (1.0 + noise * (2.0 * unit(draw(seed, (uint64_t)e)) - 1.0));
                    ++e;
                }
            }
        }
    }
    return 0;
}

extern "C" int64_t bhsp_gen_powerlaw_rows(int m, double alpha, double xmin, int max_len,
                                          double empty_frac, uint64_t seed, int* row_ptr) {
    if (m < 0 || alpha <= 1.0 || xmin <= 0 || max_len < 1 || !row_ptr) return -2;
    std::vector<int64_t> len((size_t)m);
    const double inv = -1.0 / (alpha - 1.0);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < m; ++i) {
        if (unit(draw(seed, (uint64_t)i, 7)) < empty_frac) {
            len[i] = 0;
            continue;
        }
        double l = std::floor(xmin * std::pow(unit_open0(draw(seed, (uint64_t)i, 8)), inv));
        if (!(l >= 1.0)) l = 1.0;
        if (l > max_len) l = max_len;
        len[i] = (int64_t)l;
    }
    return finish_rows(m, len, row_ptr);
}

extern "C" int64_t bhsp_gen_density_rows(int m, int n, double density, uint64_t seed, int* row_ptr) {
    if (m < 0 || n < 1 || density < 0 || !row_ptr) return -2;
    std::vector<int64_t> len((size_t)m);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < m; ++i) {
        int l = poisson((double)n * density, seed, (uint64_t)i);
        len[i] = l > n ? n : l;
    }
    return finish_rows(m, len, row_ptr);
}

extern "C" int64_t bhsp_gen_mixed_rows(int m, int n, int dense_row, double mean_len,
                                       double empty_frac, uint64_t seed, int* row_ptr) {
    if (m < 0 || n < 1 || mean_len < 0 || !row_ptr) return -2;
    std::vector<int64_t> len((size_t)m);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < m; ++i) {
        if (i == dense_row) {
            len[i] = n;
        } else if (unit(draw(seed, (uint64_t)i, 9)) < empty_frac) {
            len[i] = 0;
        } else {
            int l = poisson(mean_len, seed, (uint64_t)i);
            len[i] = l > n ? n : l;
        }
    }
    return finish_rows(m, len, row_ptr);
}

extern "C" int bhsp_gen_random_fill(int m, int n, const int* row_ptr, double lo, double hi,
                                    uint64_t seed, int* col, double* val) {
    if (m < 0 || n < 1 || !row_ptr) return -1;
    int bad = 0;
#pragma omp parallel
    {
        std::vector<int> buf;
#pragma omp for schedule(dynamic, 256) reduction(| : bad)
        for (int i = 0; i < m; ++i) {
            const int b = row_ptr[i], L = row_ptr[i + 1] - b;
            if (L <= 0) continue;
            if (L > n) {
                bad |= 1;
                continue;
            }
            int* out = col + b;
            if ((int64_t)L * 2 > n) {
                // dense-ish row: keep each column with the right selection probability
                // (selection sampling, Knuth's Algorithm S), already sorted
                int need = L, left = n, k = 0;
                for (int c = 0; c < n && need > 0; ++c, --left) {
                    if (unit(draw(seed, ((uint64_t)i << 32) | (uint32_t)c, 11)) * left < need) {
                        out[k++] = c;
                        --need;
                    }
                }
            } else {
                buf.clear();
                uint64_t k = 0;
                while ((int)buf.size() < L) {
                    const size_t old = buf.size();
                    for (int t = (int)old; t < L; ++t)
                        buf.push_back((int)(draw(seed ^ 0x1234567ull, (uint64_t)i, 16 + k++) % (uint64_t)n));
                    std::sort(buf.begin(), buf.end());
                    buf.erase(std::unique(buf.begin(), buf.end()), buf.end());
                }
                std::copy(buf.begin(), buf.end(), out);
            }
            for (int t = 0; t < L; ++t)
                val[b + t] = lo + (hi - lo) * unit(draw(seed ^ 0xABCDEF, (uint64_t)(b + t), 13));
        }
    }
    return bad ? -1 : 0;
}

extern "C" int64_t bhsp_gen_blockdiag_rows(int m, int n, int bs, int* row_ptr) {
    if (m < 0 || n < 1 || bs < 1 || !row_ptr) return -2;
    std::vector<int64_t> len((size_t)m);
    for (int i = 0; i < m; ++i) {
        const int64_t c0 = (int64_t)(i / bs) * bs;
        int64_t c1 = c0 + bs;
        if (c1 > n) c1 = n;
        len[i] = c1 > c0 ? c1 - c0 : 0;
    }
    return finish_rows(m, len, row_ptr);
}

extern "C" int bhsp_gen_blockdiag_fill(int m, int n, int bs, double lo, double hi, uint64_t seed,
                                       const int* row_ptr, int* col, double* val) {
    if (m < 0 || n < 1 || bs < 1 || !row_ptr) return -1;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < m; ++i) {
        const int c0 = (i / bs) * bs;
        int e = row_ptr[i];
        for (int c = c0; e < row_ptr[i + 1]; ++c, ++e) {
            col[e] = c;
            val[e] = lo + (hi - lo) * unit(draw(seed, (uint64_t)e, 14));
        }
    }
    return 0;
}
