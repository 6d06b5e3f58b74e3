// Seeded terrain of the benchmark scenes (host).  The reference ships only its fixed
// initVoxels world (level.cpp:82-138); the scenes at other sizes use this generator:
//   - heightfield: 2-octave value noise (periods 32 and 8, weights 1 and 1/2), heights
//     8 + floor(33 n) in [8, 40];
//   - bands below the surface: grass 3 voxels, dirt 8, stone below, with the
//     reference's base colours (grass (10,130,10), dirt (120,100,0), stone (90,90,90),
//     level.cpp:94-124) jittered by a uniform integer in [-8, 8] per channel;
//   - caves: air where 3-D value noise (period 8) exceeds 0.7;
//   - solid words 0x01000000 | rgb, air -1.
// Integer hashing (splitmix64) and float arithmetic built with -ffp-contract=off give
// the same words on every CPU.
#include <algorithm>
#include <cstdint>
#include <thread>
#include <vector>

#include "vrt_host.h"

namespace {

inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline uint64_t hash5(uint64_t seed, int64_t a, int64_t b, int64_t c, uint64_t salt) {
    uint64_t h = mix64(seed ^ (salt * 0xD1B54A32D192ED03ull));
    h = mix64(h ^ (uint64_t)a);
    h = mix64(h ^ ((uint64_t)b * 0x9E3779B97F4A7C15ull));
    h = mix64(h ^ ((uint64_t)c * 0xC2B2AE3D27D4EB4Full));
    return h;
}
inline float u01(uint64_t h) { return (float)(h >> 40) * (1.0f / 16777216.0f); }
inline float smooth(float f) { return f * f * (3.0f - 2.0f * f); }
inline float lerp(float a, float b, float t) { return a + (b - a) * t; }

float noise2(uint64_t seed, int x, int z, int P, uint64_t salt) {
    int ix = x / P, iz = z / P;
    float fx = smooth((float)(x % P) / (float)P), fz = smooth((float)(z % P) / (float)P);
    float v00 = u01(hash5(seed, ix, iz, 0, salt)), v10 = u01(hash5(seed, ix + 1, iz, 0, salt));
    float v01 = u01(hash5(seed, ix, iz + 1, 0, salt)), v11 = u01(hash5(seed, ix + 1, iz + 1, 0, salt));
    return lerp(lerp(v00, v10, fx), lerp(v01, v11, fx), fz);
}

float noise3(uint64_t seed, int x, int y, int z, int P, uint64_t salt) {
    int ix = x / P, iy = y / P, iz = z / P;
    float fx = smooth((float)(x % P) / (float)P), fy = smooth((float)(y % P) / (float)P);
    float fz = smooth((float)(z % P) / (float)P);
    float c[2][2][2];
    for (int k = 0; k < 2; k++)
        for (int j = 0; j < 2; j++)
            for (int i = 0; i < 2; i++) c[k][j][i] = u01(hash5(seed, ix + i, iy + j, iz + k, salt));
    float a0 = lerp(lerp(c[0][0][0], c[0][0][1], fx), lerp(c[0][1][0], c[0][1][1], fx), fy);
    float a1 = lerp(lerp(c[1][0][0], c[1][0][1], fx), lerp(c[1][1][0], c[1][1][1], fx), fy);
    return lerp(a0, a1, fz);
}

int column_height(uint64_t seed, int x, int z) {
    float n = (noise2(seed, x, z, 32, 1) + 0.5f * noise2(seed, x, z, 8, 2)) / 1.5f;
    int h = 8 + (int)(n * 33.0f);
    return std::min(std::max(h, 8), 40);
}

inline int jitter(int base, uint64_t h) { return std::min(255, std::max(0, base + (int)(h % 17) - 8)); }

void fill_slab(int32_t* words, int W, int H, uint64_t seed, int z0, int z1) {
    for (int z = z0; z < z1; z++)
        for (int x = 0; x < W; x++) {
            int h = std::min(column_height(seed, x, z), H);
            for (int y = 0; y < H; y++) {
                int32_t v = -1;
                if (y < h && noise3(seed, x, y, z, 8, 3) <= 0.7f) {
                    int depth = h - 1 - y;
                    int r, g, b;
                    if (depth < 3) { r = 10; g = 130; b = 10; }
                    else if (depth < 11) { r = 120; g = 100; b = 0; }
                    else { r = 90; g = 90; b = 90; }
                    r = jitter(r, hash5(seed, x, y, z, 16));
                    g = jitter(g, hash5(seed, x, y, z, 17));
                    b = jitter(b, hash5(seed, x, y, z, 18));
                    v = 0x01000000 | (r << 16) | (g << 8) | b;
                }
                words[(uint64_t)x + (uint64_t)W * y + (uint64_t)W * H * z] = v;
            }
        }
}

}  // namespace

extern "C" {

int vrt_terrain_generate(int32_t* words, int32_t W, int32_t H, uint64_t seed, int32_t threads) {
    if (!words || W < 1 || H < 1) return vrt::set_error(VRT_EINVAL, "bad terrain arguments");
    if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    threads = std::min(threads, W);
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; t++) {
        int z0 = (int)((int64_t)W * t / threads), z1 = (int)((int64_t)W * (t + 1) / threads);
        pool.emplace_back(fill_slab, words, W, H, seed, z0, z1);
    }
    for (auto& th : pool) th.join();
    return VRT_OK;
}

int vrt_terrain_height(int32_t W, uint64_t seed, int32_t x, int32_t z) {
    if (x < 0 || z < 0 || x >= W || z >= W) return vrt::set_error(VRT_EINVAL, "column outside the world");
    return column_height(seed, x, z);
}

}  // extern "C"
