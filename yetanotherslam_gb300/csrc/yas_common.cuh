// yas_common.cuh — device helpers shared by every kernel of the dense path.
//
// Contents:
//  * canonical FP32 arithmetic for the discrete decisions (block allocation,
//    visibility, pixel selection): every product and sum is rounded on its
//    own (no FMA contraction), in a fixed order, so the CPU oracle compiled
//    with -ffp-contract=off reproduces each decision bit for bit;
//  * 64-bit block keys (21-bit signed x,y,z) and the open-addressing hash
//    table of 16-byte slots that replaces the reference's bucket + excess
//    list table (RGBDFusion/utils/VoxelStructUtils.h:16-21, 173-317);
//  * the three voxel storage formats;
//  * MapDev, the by-value kernel view of one map.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include "../../include/yas.h"

namespace yas {

constexpr int kBlockSide = 8;      // voxels per block edge (VoxelMap.h:12)
constexpr int kBlockVoxels = 512;  // voxels per block (VoxelMap.h:13)
constexpr unsigned long long kEmptyKey = ~0ull;
constexpr int kMaxProbes = 2048;   // bounded linear probing (no unbounded spin)
// SMs of a GB300; grid-stride kernels size their grids in multiples of it
// (their results do not depend on the grid).
constexpr int kSMs = 152;
// Fine near-bound cells of the ray march: 2^kFineShift pixels square.
constexpr int kFineShift = 2;
constexpr int kCoordBits = 21;
constexpr int kCoordMax = (1 << (kCoordBits - 1)) - 1;   // 1048575
constexpr int kCoordMin = -(1 << (kCoordBits - 1));      // -1048576

// Sticky error bits written by kernels into MapHeader::err_bits.
__host__ __device__ constexpr unsigned err_bit(int code) { return 1u << code; }

// ------------------------------------------------------------------ FP32 canon
__device__ __forceinline__ float cmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float cadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float csub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float cdiv(float a, float b) { return __fdiv_rn(a, b); }

// Row-major rotation + translation in float (converted from a double pose on
// the host or device by round-to-nearest of each element).
struct Rigid32 {
    float r[9];
    float t[3];
};

// y = R x + t with the canonical order ((r0 x + r1 y) + r2 z) + t0.
__device__ __forceinline__ float3 rigid_exact(const Rigid32 &T, float x, float y, float z) {
    float3 o;
    o.x = cadd(cadd(cadd(cmul(T.r[0], x), cmul(T.r[1], y)), cmul(T.r[2], z)), T.t[0]);
    o.y = cadd(cadd(cadd(cmul(T.r[3], x), cmul(T.r[4], y)), cmul(T.r[5], z)), T.t[1]);
    o.z = cadd(cadd(cadd(cmul(T.r[6], x), cmul(T.r[7], y)), cmul(T.r[8], z)), T.t[2]);
    return o;
}

// Fast form (FMA allowed) for continuous quantities compared with tolerance.
__device__ __forceinline__ float3 rigid_fast(const Rigid32 &T, float x, float y, float z) {
    return make_float3(fmaf(T.r[0], x, fmaf(T.r[1], y, fmaf(T.r[2], z, T.t[0]))),
                       fmaf(T.r[3], x, fmaf(T.r[4], y, fmaf(T.r[5], z, T.t[1]))),
                       fmaf(T.r[6], x, fmaf(T.r[7], y, fmaf(T.r[8], z, T.t[2]))));
}

__device__ __forceinline__ float3 rotate_fast(const Rigid32 &T, float x, float y, float z) {
    return make_float3(fmaf(T.r[0], x, fmaf(T.r[1], y, T.r[2] * z)),
                       fmaf(T.r[3], x, fmaf(T.r[4], y, T.r[5] * z)),
                       fmaf(T.r[6], x, fmaf(T.r[7], y, T.r[8] * z)));
}

// floor division by the block side for voxel -> block, and the local index
// z*64 + y*8 + x (VoxelStructUtils.h:28-72).
__device__ __forceinline__ int floor_div8(int v) { return v >> 3; }  // arithmetic shift == floor
__device__ __forceinline__ int mod8(int v) { return v & 7; }

// ------------------------------------------------------------------ keys/hash
__host__ __device__ __forceinline__ unsigned long long pack_key(int x, int y, int z) {
    return ((unsigned long long)(x & 0x1FFFFF) << 42) | ((unsigned long long)(y & 0x1FFFFF) << 21) |
           (unsigned long long)(z & 0x1FFFFF);
}
__host__ __device__ __forceinline__ int sext21(unsigned v) {
    return (int)(v << 11) >> 11;
}
__host__ __device__ __forceinline__ void unpack_key(unsigned long long k, int &x, int &y, int &z) {
    x = sext21((unsigned)((k >> 42) & 0x1FFFFF));
    y = sext21((unsigned)((k >> 21) & 0x1FFFFF));
    z = sext21((unsigned)(k & 0x1FFFFF));
}
__host__ __device__ __forceinline__ bool coord_in_range(int x, int y, int z) {
    return x >= kCoordMin && x <= kCoordMax && y >= kCoordMin && y <= kCoordMax &&
           z >= kCoordMin && z <= kCoordMax;
}
// 64-bit finaliser of MurmurHash3 (Appleby), used as the slot hash.
__host__ __device__ __forceinline__ unsigned hash_key(unsigned long long k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ULL;
    k ^= k >> 33;
    return (unsigned)k;
}

// One hash-table slot: 16 bytes, read with a single 128-bit load.
struct __align__(16) HashSlot {
    unsigned long long key;  // kEmptyKey when free
    int ptr;                 // block index in the pool, -1 until assigned
    int pad;
};

// Device-resident counters of one map.
struct __align__(16) MapHeader {
    unsigned n_alloc;       // bump counter of the block pool (may pass max_blocks on overflow)
    unsigned n_visible;     // length of the visible list
    unsigned err_bits;      // sticky yas_status bits
    unsigned n_alloc_prev;  // n_alloc before the latest allocation pass
    unsigned n_render;      // raycast: z-range tiles written
    unsigned pad[3];
};

// ------------------------------------------------------------------ formats
template <int FMT>
struct VoxelIO;

template <>
struct VoxelIO<YAS_VOXEL_F32> {
    typedef float2 T;
    static constexpr int kBytes = 8;
    __device__ __forceinline__ static float sdf(T v) { return v.x; }
    __device__ __forceinline__ static int wt(T v) { return (int)v.y; }
    __device__ __forceinline__ static T make(float s, int w) { return make_float2(s, (float)w); }
};

// FP16 value + u8 weight, with the FP16 rounding residual in the word's spare
// byte: bits 0..15 the half h, bits 16..23 a signed residual q, bits 24..31 the
// weight.  The value's FP32 bit pattern is h's (converted exactly) plus 32 q:
// q counts 2^-18 of h's binade, 1/256 of the half's ulp, on the magnitude.  In
// the half's normal range a write therefore keeps s rounded to 18 mantissa
// bits (8 more than the half alone), so the running average's rounding stays
// ~256x smaller; a read is one conversion, one byte extract and one add.
template <>
struct VoxelIO<YAS_VOXEL_F16> {
    typedef unsigned T;
    static constexpr int kBytes = 4;
    __device__ __forceinline__ static float sdf(T v) {
        const float h = __half2float(__ushort_as_half((unsigned short)(v & 0xffffu)));
        const int q = (int)(v << 8) >> 24;
        return __int_as_float(__float_as_int(h) + q * 32);
    }
    __device__ __forceinline__ static int wt(T v) { return (int)(v >> 24); }
    __device__ __forceinline__ static T make(float s, int w) {
        unsigned short hb = __half_as_ushort(__float2half_rn(s));
        int q = 0;
        if (hb & 0x7fffu) {  // h and s share the sign; d = |s| - |h| in FP32 bit units
            const int d = (__float_as_int(s) & 0x7fffffff) -
                          (__float_as_int(__half2float(__ushort_as_half(hb))) & 0x7fffffff);
            q = (d + 16) >> 5;  // -128..128 for a normal half
            if (q > 127 && (hb & 0x7c00u)) {
                // a tie rounded down: the next half up in magnitude is 2^13
                // FP32 bit units further, so the same value is q - 256 from it
                hb = (unsigned short)(hb + 1u);
                q -= 256;
            }
            q = max(-128, min(127, q));  // clamps only below the half's normal range
        }
        return (unsigned)hb | (((unsigned)q & 0xffu) << 16) | ((unsigned)min(w, 255) << 24);
    }
};

template <>
struct VoxelIO<YAS_VOXEL_S24> {
    typedef unsigned T;
    static constexpr int kBytes = 4;
    __device__ __forceinline__ static float sdf(T v) {
        return (float)((int)v >> 8) * (1.0f / 4194304.0f);
    }
    __device__ __forceinline__ static int wt(T v) { return (int)(v & 0xffu); }
    __device__ __forceinline__ static T make(float s, int w) {
        int q = __float2int_rn(s * 4194304.0f);
        q = max(-8388608, min(8388607, q));
        return ((unsigned)q << 8) | ((unsigned)w & 0xffu);
    }
};

// The reference's voxel (VoxelMap.h:26-30: short sdf, uchar wt, padded to 4
// bytes; the word's bytes are the struct's): bits 0..15 the int16 sdf, bits
// 16..23 the weight.  PackFloat / UnPackFloat (VoxelStructUtils.h:6-14): the
// sdf is stored as (short)(s * 32767), truncated toward zero, and read back
// with an IEEE division by 32767.
template <>
struct VoxelIO<YAS_VOXEL_S16> {
    typedef unsigned T;
    static constexpr int kBytes = 4;
    __device__ __forceinline__ static float sdf(T v) {
        return __fdiv_rn((float)(short)(v & 0xffffu), 32767.0f);
    }
    __device__ __forceinline__ static int wt(T v) { return (int)((v >> 16) & 0xffu); }
    __device__ __forceinline__ static T make(float s, int w) {
        const int q = max(-32767, min(32767, __float2int_rz(__fmul_rn(s, 32767.0f))));
        return ((unsigned)q & 0xffffu) | ((unsigned)min(w, 255) << 16);
    }
};

// ------------------------------------------------------------------ map view
struct MapDev {
    HashSlot *slots;
    unsigned slot_mask;
    unsigned long long *block_keys;  // [max_blocks] key of each pool block
    void *voxels;                    // [max_blocks * 512] in the map's format
    int *visible;                    // [max_blocks] compacted visible block indices
    MapHeader *hdr;
    int max_blocks;
    float voxel_size;
    float trunc;
    float depth_min;
    float depth_max;
    int max_weight;
};

__device__ __forceinline__ unsigned num_blocks(const MapDev &m) {
    unsigned n = *(volatile unsigned *)&m.hdr->n_alloc;
    return n < (unsigned)m.max_blocks ? n : (unsigned)m.max_blocks;
}

// Read-only lookup: block index of key, or -1 (VoxelStructUtils.h:282-300).
__device__ __forceinline__ int find_block(const MapDev &m, unsigned long long key) {
    unsigned s = hash_key(key) & m.slot_mask;
#pragma unroll 1
    for (int i = 0; i < kMaxProbes; ++i) {
        ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2 *>(m.slots + s));
        if (v.x == key) return (int)(unsigned)(v.y & 0xffffffffull);
        if (v.x == kEmptyKey) return -1;
        s = (s + 1) & m.slot_mask;
    }
    return -1;
}

__device__ __forceinline__ int find_block_xyz(const MapDev &m, int bx, int by, int bz) {
    if (!coord_in_range(bx, by, bz)) return -1;
    return find_block(m, pack_key(bx, by, bz));
}

// Claims a slot for `key`: returns 1 if this call inserted it (slot index in
// *slot_out), 0 if the key was already present, -1 if the probe limit was hit.
__device__ __forceinline__ int claim_slot(const MapDev &m, unsigned long long key, unsigned *slot_out) {
    unsigned s = hash_key(key) & m.slot_mask;
#pragma unroll 1
    for (int i = 0; i < kMaxProbes; ++i) {
        unsigned long long k = __ldcg(&m.slots[s].key);
        if (k == key) return 0;
        if (k == kEmptyKey) {
            unsigned long long prev = atomicCAS(&m.slots[s].key, kEmptyKey, key);
            if (prev == kEmptyKey) {
                *slot_out = s;
                return 1;
            }
            if (prev == key) return 0;
        }
        s = (s + 1) & m.slot_mask;
    }
    return -1;
}

__device__ __forceinline__ void raise_error(const MapDev &m, int code) {
    atomicOr(&m.hdr->err_bits, err_bit(code));
}

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// Programmatic dependent launch.  A kernel launched as a dependent of the
// previous kernel on its stream may be scheduled while that kernel still runs:
// dependent_wait() returns once the previous kernel has completed and its
// writes are visible, so a dependent calls it before its first memory access.
// release_dependents() lets the next kernel's CTAs be scheduled (they still
// wait for this one to complete).  Both do nothing in a kernel launched the
// ordinary way.
__device__ __forceinline__ void dependent_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void release_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned r;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
    return r;
}

// Warp-aggregated append: every lane with `pred` gets a unique index into a
// list whose length lives at *counter; one atomicAdd per warp.  All 32 lanes
// of the warp must call it together.
__device__ __forceinline__ unsigned warp_append(unsigned *counter, bool pred) {
    unsigned mask = __ballot_sync(0xffffffffu, pred);
    if (mask == 0) return 0xffffffffu;
    int leader = __ffs(mask) - 1;
    unsigned base = 0;
    if ((int)lane_id() == leader) base = atomicAdd(counter, (unsigned)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    return pred ? base + (unsigned)__popc(mask & lanemask_lt()) : 0xffffffffu;
}

// Warp-cooperative insertion of one block key per lane (lanes with !has
// insert nothing; all 32 lanes call together): duplicates within the warp
// merge into one leader, each new key claims a hash slot (CAS), takes the
// next pool block (one atomicAdd per warp) and the warp zeroes the new blocks
// with coalesced 16-byte stores.  Table and pool exhaustion set the map's
// sticky error bits (CreateNewBlock, VoxelStructUtils.h:259-280).
template <int VBYTES>
__device__ __forceinline__ void warp_insert(const MapDev &m, unsigned long long key, bool has) {
    const unsigned lane = lane_id();
    const unsigned peers = __match_any_sync(0xffffffffu, has ? key : kEmptyKey);
    const bool leader = has && (__ffs(peers) - 1) == (int)lane;
    int claimed = 0;
    unsigned slot = 0;
    if (leader) {
        claimed = claim_slot(m, key, &slot);
        if (claimed < 0) {
            raise_error(m, YAS_ERR_TABLE_FULL);
            claimed = 0;
        }
    }
    const unsigned idx = warp_append(&m.hdr->n_alloc, claimed == 1);
    bool ok = false;
    if (claimed == 1) {
        if (idx < (unsigned)m.max_blocks) {
            m.block_keys[idx] = key;
            m.slots[slot].ptr = (int)idx;
            ok = true;
        } else {
            raise_error(m, YAS_ERR_POOL_FULL);
        }
    }
    unsigned newmask = __ballot_sync(0xffffffffu, ok);
    while (newmask) {
        const int src = __ffs(newmask) - 1;
        newmask &= newmask - 1;
        const unsigned b = __shfl_sync(0xffffffffu, idx, src);
        uint4 *dst = reinterpret_cast<uint4 *>(static_cast<char *>(m.voxels) + (size_t)b * kBlockVoxels * VBYTES);
        constexpr int n16 = kBlockVoxels * VBYTES / 16;
#pragma unroll
        for (int i = (int)lane; i < n16; i += 32) dst[i] = make_uint4(0, 0, 0, 0);
    }
}

}  // namespace yas
