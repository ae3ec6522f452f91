// wr_device.cuh — device-side data layout and arithmetic shared by the
// traversal and rendering kernels (sm_103a).
//
// Layout in HBM (one resident scene):
//   NodePair[num_pairs]  64 B each, 64-B aligned: the two children of one
//                        internal node of the reference tree — both AABBs
//                        (2 x 24 B) and both 8-byte topology words (16 B).
//                        One visit = one 64-B record = two 32-B sectors.
//   TriRec[num_slots]    48 B each: v0, v1, v2 as float4; the .w lanes carry
//                        the global triangle id, the object id and the
//                        object-local triangle id.  Slots are in leaf order,
//                        each leaf's list reversed, so that "smallest t, ties
//                        to the largest slot" reproduces the reference's
//                        tie rule (kdtree.cpp:319, 331-334).
//
// Arithmetic: all kernels are compiled with -fmad=false and IEEE div/sqrt, and
// the vector helpers keep nvVector.h's operation order, so that the traversal
// predicates are bit-identical to the reference's FP32 code.
#pragma once

#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

namespace wr {

// topology word of one child: internal -> {pair index of its children, 0};
// leaf -> {first slot, count | LEAF_FLAG}
constexpr uint32_t LEAF_FLAG = 0x80000000u;

struct __align__(64) NodePair {
    float4 a;  // L.min.x L.min.y L.min.z L.max.x
    float4 b;  // L.max.y L.max.z R.min.x R.min.y
    float4 c;  // R.min.z R.max.x R.max.y R.max.z
    uint4 t;   // L.w0 L.w1 R.w0 R.w1
};
static_assert(sizeof(NodePair) == 64, "NodePair must be 64 bytes");

struct __align__(16) TriRec {
    float4 v0;  // .w = global triangle id (bits)
    float4 v1;  // .w = object id (bits)
    float4 v2;  // .w = object-local triangle id (bits)
};
static_assert(sizeof(TriRec) == 48, "TriRec must be 48 bytes");

struct DevTree {
    const NodePair* pairs;
    const TriRec* tris;
    float root_lo[3], root_hi[3];
    uint32_t root_w0, root_w1;  // topology word of the root
    float scene_mag;            // max |coordinate| over all vertices
    uint32_t max_depth;
    uint32_t num_pairs, num_slots;
};

// Knobs of the warp-persistent traversal loop (wr_warp_trace.cuh)
struct TraceTune {
    int refill_min;  // refill idle lanes once at least this many are idle (or none is busy)
    int leaf_min;    // lanes holding postponed leaves that start the warp's leaf phase
    int steps;       // traversal steps a searching lane takes per turn of the warp loop (1..8)
};
// fastest of sweeps on GB300, kd workload: 4349 Mrays/s with one step per
// turn, 4568 with four, 4699 with six, 4673 with eight
inline TraceTune default_trace_tune() { return TraceTune{8, 8, 6}; }

struct f3 {
    float x, y, z;
};

__host__ __device__ __forceinline__ f3 mk(float x, float y, float z) { return f3{x, y, z}; }
__host__ __device__ __forceinline__ f3 operator+(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ f3 operator-(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ f3 operator-(f3 a) { return mk(-a.x, -a.y, -a.z); }
__host__ __device__ __forceinline__ f3 operator*(f3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ f3 vmul(f3 a, f3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
// nvVector.h:501-506: r = 0; r += x*x'; r += y*y'; r += z*z'
__host__ __device__ __forceinline__ float dot(f3 a, f3 b) {
    float r = 0.f;
    r += a.x * b.x;
    r += a.y * b.y;
    r += a.z * b.z;
    return r;
}
__host__ __device__ __forceinline__ f3 cross(f3 l, f3 r) {
    return mk(l.y * r.z - l.z * r.y, l.z * r.x - l.x * r.z, l.x * r.y - l.y * r.x);
}
__host__ __device__ __forceinline__ float length(f3 a) { return sqrtf(dot(a, a)); }
// vec3 / scalar leaves the vector unchanged for a zero scalar (nvVector.h:376-381)
__host__ __device__ __forceinline__ f3 divs(f3 a, float d) {
    if (d == 0.f) return a;
    return mk(a.x / d, a.y / d, a.z / d);
}
__host__ __device__ __forceinline__ f3 normalize(f3 a) {
    float r = length(a);
    if (r > 0.f) a = divs(a, r);
    return a;
}
__host__ __device__ __forceinline__ f3 xyz(float4 v) { return mk(v.x, v.y, v.z); }

// The same operations with every product and sum rounded on its own, for the
// traversal code whose results must equal the reference's FP32 bit for bit
// (box face test, triangle test, face normals, NoSelfCondition): these are
// never contracted into fused multiply-adds, whatever the compiler's -fmad
// setting, so the rest of the device code may be compiled with contraction.
#ifdef __CUDA_ARCH__
__device__ __forceinline__ float add_x(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub_x(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float mul_x(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float div_x(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float sqrt_x(float a) { return __fsqrt_rn(a); }
#else
inline float add_x(float a, float b) { return a + b; }
inline float sub_x(float a, float b) { return a - b; }
inline float mul_x(float a, float b) { return a * b; }
inline float div_x(float a, float b) { return a / b; }
inline float sqrt_x(float a) { return sqrtf(a); }
#endif
__host__ __device__ __forceinline__ f3 sub3_x(f3 a, f3 b) { return mk(sub_x(a.x, b.x), sub_x(a.y, b.y), sub_x(a.z, b.z)); }
// nvVector.h:501-506 order, unfused
__host__ __device__ __forceinline__ float dot_x(f3 a, f3 b) {
    float r = 0.f;
    r = add_x(r, mul_x(a.x, b.x));
    r = add_x(r, mul_x(a.y, b.y));
    r = add_x(r, mul_x(a.z, b.z));
    return r;
}
__host__ __device__ __forceinline__ f3 cross_x(f3 l, f3 r) {
    return mk(sub_x(mul_x(l.y, r.z), mul_x(l.z, r.y)), sub_x(mul_x(l.z, r.x), mul_x(l.x, r.z)),
              sub_x(mul_x(l.x, r.y), mul_x(l.y, r.x)));
}
__host__ __device__ __forceinline__ f3 normalize_x(f3 a) {
    const float r = sqrt_x(dot_x(a, a));
    if (r > 0.f) a = mk(div_x(a.x, r), div_x(a.y, r), div_x(a.z, r));
    return a;
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).  Draw `dim` of
// (pixel, sample) under `seed`: counter {dim/4, sample, pixel, 0}, key = seed,
// word dim%4, top 24 bits * 2^-24.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
#ifdef __CUDA_ARCH__
        uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
#else
        uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0, hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
        uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
    }
}

__host__ __device__ __forceinline__ float u24_to_float(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

// One Philox block {blk, sample, pixel, 0} under (seed_lo, seed_hi).  Not
// inlined on the device: a path draws from a dozen call sites, and one copy
// of the ten rounds keeps the shading kernels' code small.
#ifdef __CUDA_ARCH__
static __device__ __noinline__ uint4 philox_block(uint32_t blk, uint32_t sample, uint32_t pixel, uint32_t seed_lo,
                                           uint32_t seed_hi) {
    uint32_t c[4] = {blk, sample, pixel, 0u};
    philox4x32_10(c, seed_lo, seed_hi);
    return make_uint4(c[0], c[1], c[2], c[3]);
}
#else
inline uint4 philox_block(uint32_t blk, uint32_t sample, uint32_t pixel, uint32_t seed_lo, uint32_t seed_hi) {
    uint32_t c[4] = {blk, sample, pixel, 0u};
    philox4x32_10(c, seed_lo, seed_hi);
    return make_uint4(c[0], c[1], c[2], c[3]);
}
#endif

// Sequential draws of one path; keeps the four words of the current block in
// registers (selected without dynamic indexing).
struct PathRng {
    uint32_t seed_lo, seed_hi, pixel, sample, dim;
    uint32_t w0, w1, w2, w3;
    uint32_t cached_block;
    __host__ __device__ __forceinline__ void init(uint64_t seed, uint32_t px, uint32_t smp, uint32_t d0 = 0) {
        seed_lo = (uint32_t)seed;
        seed_hi = (uint32_t)(seed >> 32);
        pixel = px;
        sample = smp;
        dim = d0;
        cached_block = 0xffffffffu;
    }
    __host__ __device__ __forceinline__ float next() {
        uint32_t blk = dim >> 2;
        if (blk != cached_block) {
            const uint4 c = philox_block(blk, sample, pixel, seed_lo, seed_hi);
            w0 = c.x;
            w1 = c.y;
            w2 = c.z;
            w3 = c.w;
            cached_block = blk;
        }
        uint32_t k = dim++ & 3u;
        uint32_t w = k == 0 ? w0 : (k == 1 ? w1 : (k == 2 ? w2 : w3));
        return u24_to_float(w);
    }
};

}  // namespace wr
