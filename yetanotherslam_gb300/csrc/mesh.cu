// mesh.cu — marching-cubes extraction over every allocated block.
//
// Reference semantics (paths relative to the reference project root):
//   RGBDFusion/src/MeshEngine.cu:43-269 (MeshificationFunctor): a cube at voxel
//   p uses corners p + {0,1}^3 in the order 0:(0,0,0) 1:(1,0,0) 2:(1,1,0)
//   3:(0,1,0) 4:(0,0,1) 5:(1,0,1) 6:(1,1,1) 7:(0,1,1); all 8 must be observed
//   (weight != 0); case bit i is set when sdf_i < 0; edge vertices use the
//   reference's interpolation with its 1e-6 guards; positions are voxel
//   coordinates times the voxel size (submap metres) and every triangle carries
//   the face normal normalize((v1-v0) x (v2-v0)).
//
// The triangle table is not the reference's table (RGBDFusion/utils/
// TriangleTable.h): it is generated here from cube topology.  For each case
// the iso-contour is traced on the six faces (each face's crossings paired so
// that inside corners stay separated on ambiguous faces), the directed face
// segments are chained into loops, and each loop is fanned from its
// lowest-numbered edge.  Segment direction keeps the inside (sdf < 0) region
// on the left seen from outside the cube, which makes every triangle's normal
// point toward the inside, the same orientation as the reference table.
//
// GB300 design: one CTA per block stages the 9x9x9 sdf neighbourhood in shared
// memory (own block with 16-byte loads plus the +x/+y/+z halo from up to 7
// neighbour blocks); pass 1 counts triangles per block, a scan assigns each
// block a contiguous output range, pass 2 scans the block's cube counts and
// writes one triangle per thread, so the output order (cube order, then table
// order) is a pure function of the map.
#include <cstring>

#include "yas_internal.h"

namespace yas {

// ---------------------------------------------------------------- tables
constexpr int kMcMaxTriIdx = 31;  // up to 10 triangles + terminator

// The tables in global memory: each CTA copies them into shared memory with
// coalesced 16-byte loads (a constant-memory copy would serialise the lanes'
// distinct addresses).  g_mc_count is 0 for the cases without crossings.
__device__ __align__(16) signed char g_mc_tri[256 * kMcMaxTriIdx];
__device__ __align__(16) unsigned char g_mc_count[256];
static_assert((256 * kMcMaxTriIdx) % 16 == 0, "16-byte copies of the triangle table");

static const int kCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                  {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
static const int kEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                 {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

static int edge_of(int a, int b) {
    for (int e = 0; e < 12; ++e)
        if ((kEdge[e][0] == a && kEdge[e][1] == b) || (kEdge[e][0] == b && kEdge[e][1] == a)) return e;
    return -1;
}

// Corners of each face in counter-clockwise order about the outward normal.
static void face_ccw(int face, int out[4]) {
    // face: 0 x=0, 1 x=1, 2 y=0, 3 y=1, 4 z=0, 5 z=1
    const int axis = face / 2, side = face % 2;
    int cs[4], n = 0;
    for (int c = 0; c < 8; ++c)
        if (kCorner[c][axis] == side) cs[n++] = c;
    // order the 4 corners cyclically around the face centre
    const int u = (axis + 1) % 3, v = (axis + 2) % 3;
    int order[4] = {-1, -1, -1, -1};
    for (int i = 0; i < 4; ++i) {
        int cu = kCorner[cs[i]][u], cv = kCorner[cs[i]][v];
        int pos = (cu == 0 && cv == 0) ? 0 : (cu == 1 && cv == 0) ? 1 : (cu == 1 && cv == 1) ? 2 : 3;
        order[pos] = cs[i];
    }
    // (u, v, axis) is right-handed, so this order is CCW about +axis.
    if (side == 1) {
        for (int i = 0; i < 4; ++i) out[i] = order[i];
    } else {
        out[0] = order[0];
        out[1] = order[3];
        out[2] = order[2];
        out[3] = order[1];
    }
}

struct McTables {
    unsigned short edge[256];
    signed char tri[256][kMcMaxTriIdx];
    unsigned char count[256];
};

static void build_mc_tables(McTables &t) {
    memset(&t, 0, sizeof(t));
    memset(t.tri, -1, sizeof(t.tri));
    for (int c = 0; c < 256; ++c) {
        unsigned short em = 0;
        for (int e = 0; e < 12; ++e) {
            bool a = (c >> kEdge[e][0]) & 1, b = (c >> kEdge[e][1]) & 1;
            if (a != b) em |= (unsigned short)(1u << e);
        }
        t.edge[c] = em;
        if (em == 0) continue;
        int next[12];
        for (int e = 0; e < 12; ++e) next[e] = -1;
        for (int f = 0; f < 6; ++f) {
            int q[4];
            face_ccw(f, q);
            // crossings in CCW order: edge index and kind (+1 enter inside, -1 exit)
            int ce[4], kind[4], nc = 0;
            for (int i = 0; i < 4; ++i) {
                int a = q[i], b = q[(i + 1) & 3];
                bool ia = (c >> a) & 1, ib = (c >> b) & 1;
                if (ia != ib) {
                    ce[nc] = edge_of(a, b);
                    kind[nc] = ib ? +1 : -1;
                    ++nc;
                }
            }
            if (nc == 2) {
                int ex = kind[0] < 0 ? 0 : 1;
                next[ce[ex]] = ce[1 - ex];
            } else if (nc == 4) {
                // separate inside corners: each exit pairs with the previous enter
                for (int i = 0; i < 4; ++i)
                    if (kind[i] < 0) next[ce[i]] = ce[(i + 3) & 3];
            }
        }
        int ntri = 0, w = 0;
        bool used[12] = {false};
        for (int start = 0; start < 12; ++start) {
            if (!((em >> start) & 1) || used[start]) continue;
            int loop[12], k = 0, e = start;
            while (e >= 0 && !used[e] && k < 12) {
                used[e] = true;
                loop[k++] = e;
                e = next[e];
            }
            // fan from the lowest edge of the loop (start is the lowest unused)
            for (int i = 1; i + 1 < k; ++i) {
                t.tri[c][w++] = (signed char)loop[0];
                t.tri[c][w++] = (signed char)loop[i];
                t.tri[c][w++] = (signed char)loop[i + 1];
                ++ntri;
            }
        }
        t.count[c] = (unsigned char)ntri;
    }
}

void mesh_tables_upload() {
    static McTables tables;
    static bool built = false;
    if (!built) {
        build_mc_tables(tables);
        built = true;
    }
    unsigned char count[256];
    for (int c = 0; c < 256; ++c) count[c] = tables.edge[c] == 0 ? 0 : tables.count[c];
    cudaMemcpyToSymbol(g_mc_tri, tables.tri, sizeof(tables.tri));
    cudaMemcpyToSymbol(g_mc_count, count, sizeof(count));
    // the copies run on the legacy stream; the engines launch on
    // non-blocking streams, which do not wait for it
    cudaStreamSynchronize(cudaStreamLegacy);
}

// ---------------------------------------------------------------- staging
constexpr int kN = 9;            // staged cells per axis
constexpr int kN3 = kN * kN * kN;

// Stages block b's 9^3 neighbourhood: s[z*81 + y*9 + x] = sdf, or NaN when
// the voxel is unobserved or its block is missing.
template <int FMT>
__device__ void stage_block(const MapDev &m, int b, int bx, int by, int bz, float *s) {
    typedef VoxelIO<FMT> IO;
    const typename IO::T *vox = static_cast<const typename IO::T *>(m.voxels);
    __shared__ int nb[8];
    if (threadIdx.x < 8) {
        int c = threadIdx.x;
        nb[c] = c == 0 ? b : find_block_xyz(m, bx + (c & 1), by + ((c >> 1) & 1), bz + ((c >> 2) & 1));
    }
    __syncthreads();
    const float qnan = __int_as_float(0x7fffffff);
    // the block's own 512 voxels: 16-byte loads of consecutive words (the pool
    // is 16-byte aligned and a block's words are contiguous, z*64 + y*8 + x)
    constexpr int kPer = 16 / (int)sizeof(typename IO::T);
    const int4 *own = reinterpret_cast<const int4 *>(vox + (size_t)b * kBlockVoxels);
    for (int q = threadIdx.x; q < kBlockVoxels / kPer; q += blockDim.x) {
        const int4 w = __ldg(own + q);
        const typename IO::T *e = reinterpret_cast<const typename IO::T *>(&w);
        const int i0 = q * kPer, x = i0 & 7, y = (i0 >> 3) & 7, z = i0 >> 6;
#pragma unroll
        for (int j = 0; j < kPer; ++j) s[z * 81 + y * 9 + x + j] = IO::wt(e[j]) != 0 ? IO::sdf(e[j]) : qnan;
    }
    // the 217 halo cells (x, y or z = 8) from the +x / +y / +z neighbours
    for (int h = threadIdx.x; h < kN3 - kBlockVoxels; h += blockDim.x) {
        int x, y, z;
        if (h < 81) {  // x = 8: y, z in 0..8
            x = 8, y = h % 9, z = h / 9;
        } else if (h < 153) {  // y = 8: x in 0..7, z in 0..8
            x = (h - 81) & 7, y = 8, z = (h - 81) >> 3;
        } else {  // z = 8: x, y in 0..7
            x = (h - 153) & 7, y = (h - 153) >> 3, z = 8;
        }
        const int p = nb[(x >> 3) | ((y >> 3) << 1) | ((z >> 3) << 2)];
        float v = qnan;
        if (p >= 0) {
            const typename IO::T r = __ldg(vox + (size_t)p * kBlockVoxels + ((z & 7) << 6) + ((y & 7) << 3) + (x & 7));
            if (IO::wt(r) != 0) v = IO::sdf(r);
        }
        s[z * 81 + y * 9 + x] = v;
    }
    __syncthreads();
}

// Case index of the cube at local (x,y,z); -1 when a corner is unobserved.
__device__ __forceinline__ int cube_case(const float *s, int x, int y, int z, float sd[8]) {
    int cidx = 0;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int dx = (c == 1 || c == 2 || c == 5 || c == 6) ? 1 : 0;
        const int dy = (c == 2 || c == 3 || c == 6 || c == 7) ? 1 : 0;
        const int dz = c >= 4 ? 1 : 0;
        float v = s[(z + dz) * 81 + (y + dy) * 9 + (x + dx)];
        if (isnan(v)) return -1;
        sd[c] = v;
        if (v < 0.0f) cidx |= 1 << c;
    }
    return cidx;
}

// Triangles of a case, from a shared-memory copy of the count table (zero for
// the cases without crossings): lanes with different cases do not serialise.
__device__ __forceinline__ int cube_tris(int cidx, const unsigned char *count) {
    return cidx <= 0 ? 0 : (int)count[cidx];
}

__device__ __forceinline__ void load_counts(unsigned char *count) {
    for (int i = threadIdx.x; i < 16; i += blockDim.x)
        reinterpret_cast<int4 *>(count)[i] = reinterpret_cast<const int4 *>(g_mc_count)[i];
}

template <int FMT>
__global__ void __launch_bounds__(128) mc_count_kernel(MapDev m, unsigned nblocks, unsigned *block_tris) {
    __shared__ float s[kN3];
    __shared__ unsigned red[4];
    __shared__ __align__(16) unsigned char count[256];
    load_counts(count);  // visible after stage_block's barrier
    for (unsigned b = blockIdx.x; b < nblocks; b += gridDim.x) {
        int bx, by, bz;
        unpack_key(m.block_keys[b], bx, by, bz);
        stage_block<FMT>(m, (int)b, bx, by, bz, s);
        unsigned cnt = 0;
        for (int i = threadIdx.x; i < kBlockVoxels; i += blockDim.x) {
            float sd[8];
            cnt += cube_tris(cube_case(s, i & 7, (i >> 3) & 7, i >> 6, sd), count);
        }
        for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = cnt;
        __syncthreads();
        if (threadIdx.x == 0) block_tris[b] = red[0] + red[1] + red[2] + red[3];
        __syncthreads();
    }
}

// Exclusive scan of per-block counts (single CTA; offsets[n] = total).  Thread
// t owns the contiguous run [t * per, (t + 1) * per): it sums its run, the CTA
// scans the 1024 run sums once, and the thread writes its run's prefixes, so
// the CTA synchronises a fixed number of times whatever n is.
__global__ void __launch_bounds__(1024) scan_kernel(const unsigned *in, unsigned *out, unsigned n,
                                                    unsigned *total) {
    __shared__ unsigned warp_sums[32];
    const unsigned per = (n + blockDim.x - 1) / blockDim.x;
    const unsigned lo = min(n, threadIdx.x * per), hi = min(n, lo + per);
    unsigned sum = 0;
    for (unsigned i = lo; i < hi; ++i) sum += in[i];
    unsigned x = sum;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) >= (unsigned)o) x += y;
    }
    if ((threadIdx.x & 31) == 31) warp_sums[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
        unsigned w = warp_sums[threadIdx.x];
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, w, o);
            if (threadIdx.x >= (unsigned)o) w += y;
        }
        warp_sums[threadIdx.x] = w;
    }
    __syncthreads();
    unsigned run = x - sum + ((threadIdx.x >= 32) ? warp_sums[(threadIdx.x >> 5) - 1] : 0u);
    for (unsigned i = lo; i < hi; ++i) {
        const unsigned v = in[i];
        out[i] = run;
        run += v;
    }
    if (threadIdx.x == blockDim.x - 1) {
        const unsigned t = warp_sums[31];
        out[n] = t;
        *total = t;
    }
}

__device__ __forceinline__ float mc_interp(float v1, float v2) {
    if (fabsf(0.0f - v1) < 1e-6f) return 0.0f;
    if (fabsf(0.0f - v2) < 1e-6f) return 1.0f;
    if (fabsf(v1 - v2) < 1e-6f) return 0.0f;
    return (0.0f - v1) / (v2 - v1);
}

// Emission: one CTA per block (grid-stride), one thread per triangle.  The
// CTA stages the block's 9^3 neighbourhood, forms every cube's triangle count,
// scans the counts in cube order and lists (cube, triangle) per output slot;
// thread j then writes the block's triangles j, j + 128, ..., so consecutive
// threads write consecutive triangles.  The soup's order is cube order, then
// table order: a pure function of the map.  The triangle and
// count tables are read from shared-memory copies, so the lanes of a warp look
// up different cases without serialising on the constant cache.
constexpr int kEmitThreads = 128;
constexpr int kMaxBlockTris = kBlockVoxels * ((kMcMaxTriIdx - 1) / 3);  // 5120

// Vertex on edge e of the cube at local (lx,ly,lz), voxel position (px,py,pz),
// in voxel units: the reference's per-edge interpolation from the edge's first
// corner (MeshEngine.cu:151-225), driven by the edge and corner tables instead
// of a switch over the 12 edges, so the lanes of a warp on different edges do
// not diverge.  Along the
// edge's axis the coordinate is p + (a + t (b - a)) for corner coordinates a,
// b in {0, 1}, which is p + t or p + (1 - t) exactly as the per-edge forms.
__device__ __forceinline__ float3 edge_vertex_tab(int e, const float *s, int lx, int ly, int lz, float px, float py,
                                                  float pz) {
    // corners a, b of edge e (kEdge) as nibble e of two constants; corner c's
    // offset (kCorner): dx = bit c of 0x66, dy = bit c of 0xcc, dz = c >> 2
    const int a = (int)((0x321076543210ull >> (4 * e)) & 15ull);
    const int b = (int)((0x765447650321ull >> (4 * e)) & 15ull);
    const int ax = (0x66 >> a) & 1, ay = (0xcc >> a) & 1, az = a >> 2;
    const int bx = (0x66 >> b) & 1, by = (0xcc >> b) & 1, bz = b >> 2;
    const float va = s[(lz + az) * 81 + (ly + ay) * 9 + (lx + ax)];
    const float vb = s[(lz + bz) * 81 + (ly + by) * 9 + (lx + bx)];
    const float t = mc_interp(va, vb);
    const float ox = ax == bx ? (float)ax : (float)ax + t * (float)(bx - ax);
    const float oy = ay == by ? (float)ay : (float)ay + t * (float)(by - ay);
    const float oz = az == bz ? (float)az : (float)az + t * (float)(bz - az);
    return make_float3(px + ox, py + oy, pz + oz);
}

template <int FMT>
__global__ void __launch_bounds__(kEmitThreads) mc_emit_kernel(MapDev m, unsigned nblocks,
                                                               const unsigned *block_offset, int max_tris,
                                                               float *points, float *normals, int *cases,
                                                               int *cube_xyz) {
    __shared__ float s[kN3];
    __shared__ __align__(16) signed char tri[256][kMcMaxTriIdx];
    __shared__ __align__(16) unsigned char count[256];
    __shared__ unsigned short slot[kMaxBlockTris];  // output slot -> cube << 4 | triangle of the cube
    __shared__ unsigned char ucase[kBlockVoxels];  // case index of each cube with triangles
    __shared__ unsigned wsum[kEmitThreads / 32];
    for (int i = threadIdx.x; i < 256 * kMcMaxTriIdx / 16; i += blockDim.x)
        reinterpret_cast<int4 *>(&tri[0][0])[i] = reinterpret_cast<const int4 *>(g_mc_tri)[i];
    load_counts(count);
    const float vs = m.voxel_size;
    for (unsigned b = blockIdx.x; b < nblocks; b += gridDim.x) {
        const unsigned base = block_offset[b];
        const unsigned ntri = block_offset[b + 1] - base;
        if (ntri == 0 || base >= (unsigned)max_tris) continue;  // uniform across the CTA
        int bx, by, bz;
        unpack_key(m.block_keys[b], bx, by, bz);
        stage_block<FMT>(m, (int)b, bx, by, bz, s);  // ends with a barrier (also for the table copies)
        // triangle counts of the thread's 4 consecutive cubes, scanned over the CTA
        int cnt[4];
        unsigned mine = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int i = threadIdx.x * 4 + k;
            float sd[8];
            const int c = cube_case(s, i & 7, (i >> 3) & 7, i >> 6, sd);
            cnt[k] = cube_tris(c, count);
            ucase[i] = (unsigned char)(c < 0 ? 0 : c);
            mine += (unsigned)cnt[k];
        }
        unsigned incl = mine;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
            if ((threadIdx.x & 31) >= (unsigned)o) incl += y;
        }
        if ((threadIdx.x & 31) == 31) wsum[threadIdx.x >> 5] = incl;
        __syncthreads();
        unsigned run = incl - mine;
        for (int w = 0; w < (int)(threadIdx.x >> 5); ++w) run += wsum[w];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const unsigned i = threadIdx.x * 4 + k;
            for (int t = 0; t < cnt[k]; ++t) slot[run + t] = (unsigned short)(i << 4 | (unsigned)t);
            run += (unsigned)cnt[k];
        }
        __syncthreads();
        const unsigned nout = min(ntri, (unsigned)max_tris - base);
        for (unsigned j = threadIdx.x; j < nout; j += kEmitThreads) {
            const unsigned e = slot[j];
            const int i = (int)(e >> 4), t = (int)(e & 15u);
            const int lx = i & 7, ly = (i >> 3) & 7, lz = i >> 6;
            const int c = ucase[i];
            const int gx = bx * 8 + lx, gy = by * 8 + ly, gz = bz * 8 + lz;
            const float px = (float)gx, py = (float)gy, pz = (float)gz;
            float3 v[3];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                const float3 ev = edge_vertex_tab(tri[c][3 * t + q], s, lx, ly, lz, px, py, pz);
                v[q] = make_float3(ev.x * vs, ev.y * vs, ev.z * vs);
            }
            const float ax = v[1].x - v[0].x, ay = v[1].y - v[0].y, az = v[1].z - v[0].z;
            const float cx = v[2].x - v[0].x, cy = v[2].y - v[0].y, cz = v[2].z - v[0].z;
            float nx = ay * cz - az * cy, ny = az * cx - ax * cz, nz = ax * cy - ay * cx;
            const float nn = nx * nx + ny * ny + nz * nz;
            if (nn > 0.0f) {
                const float inv = 1.0f / sqrtf(nn);
                nx *= inv;
                ny *= inv;
                nz *= inv;
            }
            const size_t off = (size_t)base + j;
            float *pp = points + off * 9;
            float *nq = normals + off * 9;
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                pp[3 * q] = v[q].x;
                pp[3 * q + 1] = v[q].y;
                pp[3 * q + 2] = v[q].z;
                nq[3 * q] = nx;
                nq[3 * q + 1] = ny;
                nq[3 * q + 2] = nz;
            }
            cases[off] = c;
            cube_xyz[3 * off] = gx;
            cube_xyz[3 * off + 1] = gy;
            cube_xyz[3 * off + 2] = gz;
        }
        __syncthreads();
    }
}

int mesher_ensure_blocks(MeshBuffers &mb, size_t n_blocks) {
    if (mb.cap_blocks >= n_blocks) return YAS_OK;
    cudaFree(mb.block_tris);
    cudaFree(mb.block_offset);
    mb.block_tris = nullptr;
    mb.block_offset = nullptr;
    size_t cap = n_blocks < 1024 ? 1024 : n_blocks;
    if (cudaMalloc(&mb.block_tris, cap * sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc(&mb.block_offset, (cap + 1) * sizeof(unsigned)) != cudaSuccess) {
        cudaGetLastError();
        mb.cap_blocks = 0;
        return YAS_ERR_OOM;
    }
    mb.cap_blocks = cap;
    return YAS_OK;
}

int launch_meshify(const MapDev &m, int fmt, MeshBuffers &mb, unsigned n_blocks, cudaStream_t s) {
    YAS_TRY(mesher_ensure_blocks(mb, n_blocks));
    cudaMemsetAsync(mb.counters, 0, sizeof(unsigned), s);
    if (n_blocks == 0) return YAS_OK;
    const unsigned grid = n_blocks < (unsigned)kSMs * 16u ? n_blocks : (unsigned)kSMs * 16u;
    switch (fmt) {
        case YAS_VOXEL_F32:
            mc_count_kernel<YAS_VOXEL_F32><<<grid, 128, 0, s>>>(m, n_blocks, mb.block_tris);
            break;
        case YAS_VOXEL_F16:
            mc_count_kernel<YAS_VOXEL_F16><<<grid, 128, 0, s>>>(m, n_blocks, mb.block_tris);
            break;
        case YAS_VOXEL_S16:
            mc_count_kernel<YAS_VOXEL_S16><<<grid, 128, 0, s>>>(m, n_blocks, mb.block_tris);
            break;
        default:
            mc_count_kernel<YAS_VOXEL_S24><<<grid, 128, 0, s>>>(m, n_blocks, mb.block_tris);
            break;
    }
    scan_kernel<<<1, 1024, 0, s>>>(mb.block_tris, mb.block_offset, n_blocks, mb.counters);
    switch (fmt) {
        case YAS_VOXEL_F32:
            mc_emit_kernel<YAS_VOXEL_F32><<<grid, kEmitThreads, 0, s>>>(m, n_blocks, mb.block_offset, mb.max_tris,
                                                               mb.points, mb.normals, mb.cases, mb.cube_xyz);
            break;
        case YAS_VOXEL_F16:
            mc_emit_kernel<YAS_VOXEL_F16><<<grid, kEmitThreads, 0, s>>>(m, n_blocks, mb.block_offset, mb.max_tris,
                                                               mb.points, mb.normals, mb.cases, mb.cube_xyz);
            break;
        case YAS_VOXEL_S16:
            mc_emit_kernel<YAS_VOXEL_S16><<<grid, kEmitThreads, 0, s>>>(m, n_blocks, mb.block_offset, mb.max_tris,
                                                               mb.points, mb.normals, mb.cases, mb.cube_xyz);
            break;
        default:
            mc_emit_kernel<YAS_VOXEL_S24><<<grid, kEmitThreads, 0, s>>>(m, n_blocks, mb.block_offset, mb.max_tris,
                                                               mb.points, mb.normals, mb.cases, mb.cube_xyz);
            break;
    }
    return YAS_OK;
}

}  // namespace yas

// Host-visible table access for tests (same generator as the device tables).
extern "C" YAS_API int yas_mc_tables(unsigned short *edge, signed char *tri, unsigned char *count) {
    yas::McTables t;
    yas::build_mc_tables(t);
    if (edge) memcpy(edge, t.edge, sizeof(t.edge));
    if (tri) memcpy(tri, t.tri, sizeof(t.tri));
    if (count) memcpy(count, t.count, sizeof(t.count));
    return YAS_OK;
}
