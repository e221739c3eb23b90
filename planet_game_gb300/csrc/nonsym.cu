// The non-symmetric transport solves on a planet's transport graph, on the GPU:
//
//  - block ILU(0) (sim/core/math/incomplete_lu.cpp): factorisation and triangular solves
//    level-scheduled inside each block (one CTA per block, the rows of a dependency
//    level in parallel), the same operations in the same order as the reference's, so
//    the factor and its solves are bit-identical;
//  - right-preconditioned BiCGSTAB as the reference's (heat_transport.cpp:823-897), x0 = 0,
//    shadow = r0, its breakdown tests; dots are fixed-order device reductions;
//  - advection_diffusion_source (heat_transport.cpp:774-815), bit-identical;
//  - solve_implicit_tracer (heat_transport.cpp:901-1081): the stacked layers' implicit
//    upwind/eddy/vertical system, BiCGSTAB with the stacked block ILU(0), the flux form
//    of the solution accumulated per row in the reference's order;
//  - solve_implicit_advection_diffusion (heat_transport.cpp:1083-1318): Newton on h with
//    the Jacobian on the graph's pattern, BiCGSTAB preconditioned by the V-cycle of the
//    eddies' symmetric part followed by the block ILU(0) of the full Jacobian on what is
//    left, and the line search of the implicit transport solve.
//
// Compiled without FMA contraction: every expression rounds as the reference's does.
#include "../../include/planetsim_gb300.h"
#include "capi_internal.hpp"
#include "host/ilu_pattern.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <functional>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <utility>
#include <vector>

namespace psgb {

namespace {

constexpr int kThreads = 256;
constexpr int kIluThreads = 128;

unsigned blocks_of(std::size_t n) { return static_cast<unsigned>((n + kThreads - 1) / kThreads); }

// std::max(a, b): b if a < b, else a (NaN in `a` kept, as the reference's).
__device__ __forceinline__ double std_max(double a, double b) { return a < b ? b : a; }

void require(bool ok, const char* what) {
    if (!ok) throw std::invalid_argument(what);
}

#define PSGB_CHECK_LAUNCH() PSGB_CUDA(cudaGetLastError())

// ---- block ILU(0) -------------------------------------------------------------------

struct IluView {
    const std::uint32_t *start, *column, *diagonal, *update_start, *update_t, *update_at;
    const std::int32_t* source;
    const std::uint32_t *lo_block, *lo_level, *lo_order, *up_block, *up_level, *up_order;
    double* value;
    int* flag;
    std::uint32_t rows;
};

// value = the matrix on the pattern: diagonal * scale, off-diagonals from their CSR entries.
__global__ void k_ilu_load(IluView v, const double* __restrict__ diag, const double* __restrict__ off, double scale) {
    const std::uint32_t i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= v.rows) return;
    for (std::uint32_t q = v.start[i]; q < v.start[i + 1]; ++q) {
        const std::int32_t k = v.source[q];
        v.value[q] = k < 0 ? diag[i] * scale : off[k];
    }
}

// IKJ elimination restricted to the pattern (incomplete_lu.cpp:108-135), a level at a time.
__global__ void __launch_bounds__(kIluThreads) k_ilu_factor(IluView v) {
    const std::uint32_t b = blockIdx.x;
    for (std::uint32_t lv = v.lo_block[b]; lv < v.lo_block[b + 1]; ++lv) {
        for (std::uint32_t idx = v.lo_level[lv] + threadIdx.x; idx < v.lo_level[lv + 1]; idx += kIluThreads) {
            const std::uint32_t i = v.lo_order[idx];
            for (std::uint32_t q = v.start[i]; q < v.diagonal[i]; ++q) {
                const double pivot = v.value[v.diagonal[v.column[q]]];
                if (pivot == 0.0) atomicExch(v.flag, 1);   // the reference throws here
                const double lq = v.value[q] / pivot;
                v.value[q] = lq;
                for (std::uint32_t u = v.update_start[q]; u < v.update_start[q + 1]; ++u)
                    v.value[v.update_at[u]] -= lq * v.value[v.update_t[u]];
            }
        }
        __syncthreads();
    }
}

// x <- (LU)^-1 x (incomplete_lu.cpp:137-152): forward, then backward, level by level.
__global__ void __launch_bounds__(kIluThreads) k_ilu_solve(IluView v, double* __restrict__ x) {
    const std::uint32_t b = blockIdx.x;
    for (std::uint32_t lv = v.lo_block[b]; lv < v.lo_block[b + 1]; ++lv) {
        for (std::uint32_t idx = v.lo_level[lv] + threadIdx.x; idx < v.lo_level[lv + 1]; idx += kIluThreads) {
            const std::uint32_t i = v.lo_order[idx];
            double sum = x[i];
            for (std::uint32_t q = v.start[i]; q < v.diagonal[i]; ++q) sum -= v.value[q] * x[v.column[q]];
            x[i] = sum;
        }
        __syncthreads();
    }
    for (std::uint32_t lv = v.up_block[b]; lv < v.up_block[b + 1]; ++lv) {
        for (std::uint32_t idx = v.up_level[lv] + threadIdx.x; idx < v.up_level[lv + 1]; idx += kIluThreads) {
            const std::uint32_t i = v.up_order[idx];
            double sum = x[i];
            for (std::uint32_t q = v.diagonal[i] + 1; q < v.start[i + 1]; ++q) sum -= v.value[q] * x[v.column[q]];
            x[i] = sum / v.value[v.diagonal[i]];
        }
        __syncthreads();
    }
}

// The triangular solves with the block's x in shared memory and per-level records (the
// row, its couplings' block-local columns and their factor values packed next to them):
// a thread owns one row of a level, loads the next level's record before the current
// level's barrier, so a level costs a barrier and shared-memory reads rather than a chain
// of dependent global loads. Same terms in the same order as k_ilu_solve: same bits.
struct IluRecords {
    const std::uint16_t* row;
    const std::uint8_t* count;
    const std::uint16_t* col;      // [rows][8]
    const std::uint32_t* q;        // [rows][8]: value positions
    double* val;                   // [rows][8]: packed values
    const std::uint32_t* dq;       // upper: the row's diagonal position
    double* dval;                  // upper: the diagonal value
    const std::uint32_t* block;    // [blocks + 1] levels
    const std::uint32_t* level;    // [levels + 1]
};

struct IluShared {
    IluRecords lo, up;
    const std::uint32_t* block_start;   // [blocks + 1] rows
};

__global__ void k_ilu_pack(std::uint32_t rows, IluShared s, const double* __restrict__ value) {
    const std::uint32_t idx = blockIdx.x * kThreads + threadIdx.x;
    if (idx >= rows) return;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        s.lo.val[idx * 8 + k] = k < s.lo.count[idx] ? value[s.lo.q[idx * 8 + k]] : 0.0;
        s.up.val[idx * 8 + k] = k < s.up.count[idx] ? value[s.up.q[idx * 8 + k]] : 0.0;
    }
    s.up.dval[idx] = value[s.up.dq[idx]];
}

struct Rec {
    int row, count;
    std::uint16_t col[8];
    double val[8];
    double diag;
};

__device__ __forceinline__ Rec load_rec(const IluRecords& r, std::uint32_t lv, bool upper) {
    Rec x;
    x.row = -1;
    x.count = 0;
    x.diag = 1.0;
    const std::uint32_t idx = r.level[lv] + threadIdx.x;
    if (idx < r.level[lv + 1]) {
        x.row = r.row[idx];
        x.count = r.count[idx];
        const uint4 c = *reinterpret_cast<const uint4*>(r.col + std::size_t(idx) * 8);
        const std::uint16_t* cc = reinterpret_cast<const std::uint16_t*>(&c);
#pragma unroll
        for (int k = 0; k < 8; ++k) x.col[k] = cc[k];
        const double2* v = reinterpret_cast<const double2*>(r.val + std::size_t(idx) * 8);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const double2 d = v[k];
            x.val[2 * k] = d.x;
            x.val[2 * k + 1] = d.y;
        }
        if (upper) x.diag = r.dval[idx];
    }
    return x;
}

constexpr unsigned kIluSharedThreads = 512;   // the widest level the shared-memory solve takes

__global__ void __launch_bounds__(kIluSharedThreads, 1) k_ilu_solve_shared(IluShared s, double* __restrict__ x) {
    extern __shared__ double xs[];
    const std::uint32_t b = blockIdx.x;
    const std::uint32_t first = s.block_start[b], n = s.block_start[b + 1] - first;
    for (std::uint32_t r = threadIdx.x; r < n; r += blockDim.x) xs[r] = x[first + r];
    __syncthreads();
    for (int part = 0; part < 2; ++part) {
        const bool upper = part == 1;
        const IluRecords& R = upper ? s.up : s.lo;
        const std::uint32_t lv0 = R.block[b], lv1 = R.block[b + 1];
        const Rec none{-1, 0, {}, {}, 1.0};
        // the next level's record loads while this level computes and meets
        Rec cur = lv0 < lv1 ? load_rec(R, lv0, upper) : none;
        for (std::uint32_t lv = lv0; lv < lv1; ++lv) {
            const Rec next = lv + 1 < lv1 ? load_rec(R, lv + 1, upper) : none;
            if (cur.row >= 0) {
                double sum = xs[cur.row];
#pragma unroll
                for (int k = 0; k < 8; ++k)
                    if (k < cur.count) sum -= cur.val[k] * xs[cur.col[k]];
                xs[cur.row] = upper ? sum / cur.diag : sum;
            }
            __syncthreads();
            cur = next;
        }
    }
    for (std::uint32_t r = threadIdx.x; r < n; r += blockDim.x) x[first + r] = xs[r];
}

}  // namespace

// A block ILU(0) structure on the device, its values refactored per matrix.
class DeviceIlu {
  public:
    explicit DeviceIlu(const IluPattern& p) : rows_(p.rows), blocks_(p.blocks) {
        v_.start = store_.upload(p.start);
        v_.column = store_.upload(p.column);
        v_.diagonal = store_.upload(p.diagonal);
        v_.update_start = store_.upload(p.update_start);
        v_.update_t = store_.upload(p.update_t);
        v_.update_at = store_.upload(p.update_at);
        v_.source = store_.upload(p.source);
        v_.lo_block = store_.upload(p.lower.block_level);
        v_.lo_level = store_.upload(p.lower.level_start);
        v_.lo_order = store_.upload(p.lower.order);
        v_.up_block = store_.upload(p.upper.block_level);
        v_.up_level = store_.upload(p.upper.level_start);
        v_.up_order = store_.upload(p.upper.order);
        v_.value = store_.alloc<double>(p.column.size());
        v_.flag = store_.alloc<int>(1);
        v_.rows = p.rows;
        // the shared-memory solve, when the pattern has its records and a level fits a block
        const std::uint32_t widest = std::max(p.lower.widest, p.upper.widest);
        if (!p.lower.rec_row.empty() && widest <= kIluSharedThreads) {
            auto records = [&](const LevelSchedule& sch, bool upper) {
                IluRecords r{};
                r.row = store_.upload(sch.rec_row);
                r.count = store_.upload(sch.rec_count);
                r.col = store_.upload(sch.rec_col);
                r.q = store_.upload(sch.rec_q);
                r.val = store_.alloc<double>(sch.rec_q.size());
                r.block = upper ? v_.up_block : v_.lo_block;
                r.level = upper ? v_.up_level : v_.lo_level;
                if (upper) {
                    std::vector<std::uint32_t> dq(p.rows);
                    for (std::uint32_t idx = 0; idx < p.rows; ++idx) dq[idx] = p.diagonal[sch.order[idx]];
                    r.dq = store_.upload(dq);
                    r.dval = store_.alloc<double>(p.rows);
                }
                return r;
            };
            shared_.lo = records(p.lower, false);
            shared_.up = records(p.upper, true);
            std::uint32_t most = 0;
            std::vector<std::uint32_t> starts(p.blocks + 1, 0);
            for (std::uint32_t b = 0; b < p.blocks; ++b) {
                // block b's rows: the lower schedule lists them level by level
                const std::uint32_t lv0 = p.lower.block_level[b], lv1 = p.lower.block_level[b + 1];
                const std::uint32_t count = lv1 > lv0 ? p.lower.level_start[lv1] - p.lower.level_start[lv0] : 0;
                starts[b + 1] = starts[b] + count;
                most = std::max(most, count);
            }
            shared_.block_start = store_.upload(starts);
            shared_threads_ = std::max(32u, (widest + 31) / 32 * 32);
            shared_bytes_ = std::max<std::size_t>(8, std::size_t(most) * sizeof(double));
            use_shared_ = shared_bytes_ <= 48 * 1024 ||
                          cudaFuncSetAttribute(k_ilu_solve_shared, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               static_cast<int>(shared_bytes_)) == cudaSuccess;
            cudaGetLastError();
        }
    }

    // Factors diag * scale + off (CSR entries as the pattern's source); throws Breakdown
    // on a zero pivot, where the reference throws std::runtime_error.
    void factor(const double* diag, const double* off, double scale, cudaStream_t st) {
        PSGB_CUDA(cudaMemsetAsync(v_.flag, 0, sizeof(int), st));
        k_ilu_load<<<blocks_of(rows_), kThreads, 0, st>>>(v_, diag, off, scale);
        PSGB_CHECK_LAUNCH();
        k_ilu_factor<<<blocks_, kIluThreads, 0, st>>>(v_);
        PSGB_CHECK_LAUNCH();
        if (use_shared_) {
            k_ilu_pack<<<blocks_of(rows_), kThreads, 0, st>>>(rows_, shared_, v_.value);
            PSGB_CHECK_LAUNCH();
        }
        int flag = 0;
        PSGB_CUDA(cudaMemcpyAsync(&flag, v_.flag, sizeof(int), cudaMemcpyDeviceToHost, st));
        PSGB_CUDA(cudaStreamSynchronize(st));
        if (flag != 0) throw Breakdown("incomplete LU: zero pivot");
    }

    void solve(double* x, cudaStream_t st) const {
        if (use_shared_) {
            k_ilu_solve_shared<<<blocks_, shared_threads_, shared_bytes_, st>>>(shared_, x);
        } else {
            k_ilu_solve<<<blocks_, kIluThreads, 0, st>>>(v_, x);
        }
        PSGB_CHECK_LAUNCH();
    }

    std::uint32_t rows() const { return rows_; }

  private:
    DeviceStore store_;
    IluView v_{};
    std::uint32_t rows_, blocks_;
    IluShared shared_{};
    bool use_shared_ = false;
    unsigned shared_threads_ = 0;
    std::size_t shared_bytes_ = 0;
};

namespace {

// ---- reductions and BiCGSTAB -------------------------------------------------------

// Fixed-order block sum (256 threads): a butterfly in each warp, then one over the eight
// warp sums; the same bits on every run.
__device__ double tree_sum(double v, double* sh) {
    const int t = threadIdx.x;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((t & 31) == 0) sh[t >> 5] = v;
    __syncthreads();
    double r = (t & 31) < kThreads / 32 ? sh[t & 31] : 0.0;
    if (t < 32) {
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
        if (t == 0) sh[32] = r;
    }
    __syncthreads();
    r = sh[32];
    __syncthreads();
    return r;
}
__device__ double tree_max(double v, double* sh) {
    const int t = threadIdx.x;
    sh[t] = v;
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1) {
        if (t < s) sh[t] = fmax(sh[t], sh[t + s]);
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

constexpr int kQ = 4;   // quantities per block partial

// Block partials of up to two dots: u1.v1, u2.v2 (u2 null: one).
__global__ void __launch_bounds__(kThreads) k_dots(std::uint32_t n, const double* __restrict__ u1,
                                                   const double* __restrict__ v1, const double* __restrict__ u2,
                                                   const double* __restrict__ v2, double* __restrict__ partial) {
    __shared__ double sh[kThreads];
    const std::uint32_t i = blockIdx.x * kThreads + threadIdx.x;
    const double a = i < n ? u1[i] * v1[i] : 0.0;
    const double s1 = tree_sum(a, sh);
    double s2 = 0.0;
    if (u2 != nullptr) s2 = tree_sum(i < n ? u2[i] * v2[i] : 0.0, sh);
    if (threadIdx.x == 0) {
        partial[blockIdx.x * kQ + 0] = s1;
        partial[blockIdx.x * kQ + 1] = s2;
    }
}

// One block: the partials of `quantities` values in fixed order; bit q of max_mask: a max.
__global__ void __launch_bounds__(kThreads) k_finish(unsigned blocks, int quantities, unsigned max_mask,
                                                     const double* __restrict__ partial, double* __restrict__ out) {
    __shared__ double sh[kThreads];
    for (int q = 0; q < quantities; ++q) {
        const bool is_max = (max_mask >> q) & 1u;
        double v = 0.0;
        for (unsigned b = threadIdx.x; b < blocks; b += kThreads) {
            const double x = partial[b * kQ + q];
            v = is_max ? fmax(v, x) : v + x;
        }
        const double r = is_max ? tree_max(v, sh) : tree_sum(v, sh);
        if (threadIdx.x == 0) out[q] = r;
    }
}

__global__ void k_copy(std::uint32_t n, const double* __restrict__ a, double* __restrict__ b) {
    const std::uint32_t i = blockIdx.x * kThreads + threadIdx.x;
    if (i < n) b[i] = a[i];
}
__global__ void k_bicg_p(std::uint32_t n, const double* __restrict__ r, double* __restrict__ p,
                         const double* __restrict__ v, double beta, double omega) {
    const std::uint32_t i = blockIdx.x * kThreads + threadIdx.x;
    if (i < n) p[i] = r[i] + beta * (p[i] - omega * v[i]);
}
__global__ void k_bicg_s(std::uint32_t n, const double* __restrict__ r, const double* __restrict__ v, double alpha,
                         double* __restrict__ s) {
    const std::uint32_t i = blockIdx.x * kThreads + threadIdx.x;
    if (i < n) s[i] = r[i] - alpha * v[i];
}
__global__ void k_bicg_x1(std::uint32_t n, double* __restrict__ x, const double* __restrict__ p_hat, double alpha) {
    const std::uint32_t i = blockIdx.x * kThreads + threadIdx.x;
    if (i < n) x[i] += alpha * p_hat[i];
}
__global__ void k_bicg_xr(std::uint32_t n, double* __restrict__ x, double* __restrict__ r,
                          const double* __restrict__ p_hat, const double* __restrict__ s_hat,
                          const double* __restrict__ s, const double* __restrict__ t, double alpha, double omega) {
    const std::uint32_t i = blockIdx.x * kThreads + threadIdx.x;
    if (i < n) {
        x[i] += alpha * p_hat[i] + omega * s_hat[i];
        r[i] = s[i] - omega * t[i];
    }
}


// y = diag x + off x (the reference's apply) on an ELL copy of the off-diagonals (slot-major,
// coalesced): slot j of row r is CSR entry offset[r] + j, so the terms add in the same
// order, the same bits.
struct Ell {
    std::uint32_t rows, width;
    const std::uint8_t* degree;     // [rows]
    const std::uint32_t* col;       // [width][rows]
};

__global__ void k_csr_to_ell(Ell e, const std::uint32_t* __restrict__ offset, const double* __restrict__ off,
                             double* __restrict__ val) {
    const std::uint32_t r = blockIdx.x * kThreads + threadIdx.x;
    if (r >= e.rows) return;
    const std::uint32_t first = offset[r], deg = e.degree[r];
    for (std::uint32_t j = 0; j < e.width; ++j) val[std::size_t(j) * e.rows + r] = j < deg ? off[first + j] : 0.0;
}

__global__ void k_ell_apply(Ell e, const double* __restrict__ val, const double* __restrict__ diag,
                            const double* __restrict__ x, double* __restrict__ y) {
    const std::uint32_t r = blockIdx.x * kThreads + threadIdx.x;
    if (r >= e.rows) return;
    const std::uint32_t deg = e.degree[r];
    double sum = diag[r] * x[r];
    for (std::uint32_t j = 0; j < e.width; ++j) {
        if (j < deg) sum += val[std::size_t(j) * e.rows + r] * x[e.col[std::size_t(j) * e.rows + r]];
    }
    y[r] = sum;
}

// Device scratch and the scalars read back for the host's decisions.
class Scalars {
  public:
    Scalars(DeviceStore& store, std::size_t n) : blocks_(blocks_of(n)), n_(n) {
        partial_ = store.alloc<double>(std::size_t(blocks_) * kQ);
        out_ = store.alloc<double>(kQ);
        host_.reset(kQ);
    }
    // u1.v1 (and u2.v2)
    std::pair<double, double> dots(const double* u1, const double* v1, const double* u2, const double* v2,
                                   cudaStream_t st) {
        k_dots<<<blocks_, kThreads, 0, st>>>(static_cast<std::uint32_t>(n_), u1, v1, u2, v2, partial_);
        PSGB_CHECK_LAUNCH();
        return read(u2 != nullptr ? 2 : 1, 0u, st);
    }
    double* partial() { return partial_; }
    unsigned blocks() const { return blocks_; }
    // Finishes `q` partials already written.
    std::pair<double, double> read(int q, unsigned max_mask, cudaStream_t st) {
        k_finish<<<1, kThreads, 0, st>>>(blocks_, q, max_mask, partial_, out_);
        PSGB_CHECK_LAUNCH();
        PSGB_CUDA(cudaMemcpyAsync(host_.data(), out_, q * sizeof(double), cudaMemcpyDeviceToHost, st));
        PSGB_CUDA(cudaStreamSynchronize(st));
        return {host_.data()[0], q > 1 ? host_.data()[1] : 0.0};
    }

  private:
    unsigned blocks_;
    std::size_t n_;
    double* partial_;
    double* out_;
    PinnedDoubles host_;
};

using Op = std::function<void(const double*, double*)>;

// BiCGSTAB's vectors, allocated once per solve.
struct BicgWork {
    double *r, *shadow, *p, *v, *p_hat, *s, *s_hat, *t;
    BicgWork(DeviceStore& store, std::size_t n)
        : r(store.alloc<double>(n)), shadow(store.alloc<double>(n)), p(store.alloc<double>(n)),
          v(store.alloc<double>(n)), p_hat(store.alloc<double>(n)), s(store.alloc<double>(n)),
          s_hat(store.alloc<double>(n)), t(store.alloc<double>(n)) {}
};

// Right-preconditioned BiCGSTAB (heat_transport.cpp:823-897): x <- A^-1 b from x = 0.
int bicgstab(std::size_t n, const Op& apply, const Op& precondition, const double* b, double* x, double tolerance,
             int max_iterations, const BicgWork& work, Scalars& sc, cudaStream_t st) {
    const std::uint32_t un = static_cast<std::uint32_t>(n);
    const unsigned g = blocks_of(n);
    double *r = work.r, *shadow = work.shadow, *p = work.p, *v = work.v, *p_hat = work.p_hat, *s = work.s,
           *s_hat = work.s_hat, *t = work.t;
    PSGB_CUDA(cudaMemsetAsync(x, 0, n * 8, st));
    k_copy<<<g, kThreads, 0, st>>>(un, b, r);
    k_copy<<<g, kThreads, 0, st>>>(un, b, shadow);
    PSGB_CUDA(cudaMemsetAsync(p, 0, n * 8, st));
    PSGB_CUDA(cudaMemsetAsync(v, 0, n * 8, st));
    PSGB_CHECK_LAUNCH();
    const double b_norm = std::sqrt(sc.dots(b, b, nullptr, nullptr, st).first);
    if (!(b_norm > 0.0)) return 0;
    double rho = 1.0, alpha = 1.0, omega = 1.0;
    int iteration = 0;
    while (iteration < max_iterations) {
        const double rho_next = sc.dots(shadow, r, nullptr, nullptr, st).first;
        if (rho_next == 0.0 || omega == 0.0) break;
        const double beta = rho_next / rho * (alpha / omega);
        rho = rho_next;
        k_bicg_p<<<g, kThreads, 0, st>>>(un, r, p, v, beta, omega);
        PSGB_CHECK_LAUNCH();
        precondition(p, p_hat);
        apply(p_hat, v);
        const double shadow_v = sc.dots(shadow, v, nullptr, nullptr, st).first;
        if (shadow_v == 0.0) break;
        alpha = rho / shadow_v;
        k_bicg_s<<<g, kThreads, 0, st>>>(un, r, v, alpha, s);
        PSGB_CHECK_LAUNCH();
        ++iteration;
        if (std::sqrt(sc.dots(s, s, nullptr, nullptr, st).first) <= tolerance * b_norm) {
            k_bicg_x1<<<g, kThreads, 0, st>>>(un, x, p_hat, alpha);
            PSGB_CHECK_LAUNCH();
            break;
        }
        precondition(s, s_hat);
        apply(s_hat, t);
        const auto [t_t, t_s] = sc.dots(t, t, t, s, st);
        omega = t_t > 0.0 ? t_s / t_t : 0.0;
        k_bicg_xr<<<g, kThreads, 0, st>>>(un, x, r, p_hat, s_hat, s, t, alpha, omega);
        PSGB_CHECK_LAUNCH();
        if (std::sqrt(sc.dots(r, r, nullptr, nullptr, st).first) <= tolerance * b_norm) break;
    }
    return iteration;
}

// ---- advection-diffusion source ----------------------------------------------------

struct Transport {
    std::uint32_t layers;
    const double* conductance;   // [entries]
    const double* outflow;       // [layers][entries]
    const double* latent;        // [nodes] or null
    double heat_capacity;
};

struct GraphView {
    std::uint32_t nodes, entries;
    const std::uint32_t* offset;
    const std::uint32_t* neighbour;
    const double* area;
};

// H_eddy and H_advective per node (heat_transport.cpp:795-813).
__global__ void k_advection_source(GraphView g, Transport tr, const double* __restrict__ mean,
                                   const double* __restrict__ energy, double* __restrict__ eddy_out,
                                   double* __restrict__ advective_out) {
    const std::uint32_t a = blockIdx.x * kThreads + threadIdx.x;
    if (a >= g.nodes) return;
    double eddy = 0.0, advective = 0.0;
    for (std::uint32_t k = g.offset[a]; k < g.offset[a + 1]; ++k) {
        const std::uint32_t b = g.neighbour[k];
        eddy += tr.conductance[k] * (mean[b] - mean[a]);
        for (std::uint32_t l = 0; l < tr.layers; ++l) {
            const double out = tr.outflow[std::size_t(l) * g.entries + k];
            const std::uint32_t upwind = out > 0.0 ? a : b;
            advective -= out * energy[std::size_t(l) * g.nodes + upwind];
        }
    }
    double e = eddy / g.area[a];
    if (tr.latent != nullptr) e -= tr.latent[a];
    eddy_out[a] = e;
    advective_out[a] = advective / g.area[a];
}

// F = h - (H_eddy + H_adv) and the block partials of sum A F^2 and max |F|.
__global__ void __launch_bounds__(kThreads) k_advection_residual(GraphView g, const double* __restrict__ h,
                                                                 const double* __restrict__ eddy,
                                                                 const double* __restrict__ advective,
                                                                 double* __restrict__ residual,
                                                                 double* __restrict__ partial) {
    __shared__ double sh[kThreads];
    const std::uint32_t a = blockIdx.x * kThreads + threadIdx.x;
    double merit = 0.0, largest = 0.0;
    if (a < g.nodes) {
        const double r = h[a] - (eddy[a] + advective[a]);
        residual[a] = r;
        merit = g.area[a] * r * r;
        largest = fabs(r);
    }
    const double s = tree_sum(merit, sh);
    const double m = tree_max(largest, sh);
    if (threadIdx.x == 0) {
        partial[blockIdx.x * kQ + 0] = s;
        partial[blockIdx.x * kQ + 1] = m;
    }
}

// The Newton matrix J = I - dH/dh on the graph's pattern and the right-hand side -F
// (heat_transport.cpp:1171-1195); the V-cycle's symmetric matrix A/theta' + K
// (heat_transport.cpp:1220-1232).
__global__ void k_advection_jacobian(GraphView g, Transport tr, const double* __restrict__ slope,
                                     const double* __restrict__ energy_slope, const double* __restrict__ residual,
                                     double* __restrict__ diagonal, double* __restrict__ off, double* __restrict__ rhs,
                                     double* __restrict__ sym_diagonal, double* __restrict__ sym_off) {
    const std::uint32_t a = blockIdx.x * kThreads + threadIdx.x;
    if (a >= g.nodes) return;
    const double inverse_area = 1.0 / g.area[a];
    double own = 0.0, conductance_sum = 0.0;
    for (std::uint32_t k = g.offset[a]; k < g.offset[a + 1]; ++k) {
        const std::uint32_t b = g.neighbour[k];
        const double G = tr.conductance[k];
        own -= G * slope[a];
        double neighbour = G * slope[b];
        for (std::uint32_t l = 0; l < tr.layers; ++l) {
            const double out = tr.outflow[std::size_t(l) * g.entries + k];
            if (out > 0.0) {
                own -= out * energy_slope[std::size_t(l) * g.nodes + a];
            } else {
                neighbour -= out * energy_slope[std::size_t(l) * g.nodes + b];
            }
        }
        off[k] = -neighbour * inverse_area;
        conductance_sum += G;
        sym_off[k] = -G;
    }
    diagonal[a] = 1.0 - own * inverse_area;
    rhs[a] = -residual[a];
    sym_diagonal[a] = g.area[a] / std_max(slope[a], 1.0e-12) + conductance_sum;
}

// scaled = A x
__global__ void k_scale_area(std::uint32_t n, const double* __restrict__ area, const double* __restrict__ x,
                             double* __restrict__ out) {
    const std::uint32_t a = blockIdx.x * kThreads + threadIdx.x;
    if (a < n) out[a] = area[a] * x[a];
}
// y /= max(theta', 1e-12)
__global__ void k_unscale_slope(std::uint32_t n, const double* __restrict__ slope, double* __restrict__ y) {
    const std::uint32_t a = blockIdx.x * kThreads + threadIdx.x;
    if (a < n) y[a] /= std_max(slope[a], 1.0e-12);
}
// leftover = x - leftover
__global__ void k_leftover(std::uint32_t n, const double* __restrict__ x, double* __restrict__ leftover) {
    const std::uint32_t a = blockIdx.x * kThreads + threadIdx.x;
    if (a < n) leftover[a] = x[a] - leftover[a];
}
__global__ void k_add(std::uint32_t n, const double* __restrict__ d, double* __restrict__ y) {
    const std::uint32_t a = blockIdx.x * kThreads + threadIdx.x;
    if (a < n) y[a] += d[a];
}
// h0 = max(initial, floor) or max(0, floor)
__global__ void k_advection_start(std::uint32_t n, const double* __restrict__ initial, const double* __restrict__ floor,
                                  double* __restrict__ h) {
    const std::uint32_t a = blockIdx.x * kThreads + threadIdx.x;
    if (a >= n) return;
    h[a] = initial != nullptr ? std_max(initial[a], floor[a]) : std_max(0.0, floor[a]);
}
// trial = max(h + step delta, floor)
__global__ void k_advection_trial(std::uint32_t n, const double* __restrict__ h, const double* __restrict__ delta,
                                  double step, const double* __restrict__ floor, double* __restrict__ trial) {
    const std::uint32_t a = blockIdx.x * kThreads + threadIdx.x;
    if (a >= n) return;
    trial[a] = std_max(h[a] + step * delta[a], floor[a]);
}
// H = eddy + advective and the block partials of sum A H, sum A|H|, sum A|H_eddy|, sum A|H_adv|
__global__ void __launch_bounds__(kThreads) k_advection_final(GraphView g, const double* __restrict__ eddy,
                                                              const double* __restrict__ advective,
                                                              double* __restrict__ out, double* __restrict__ partial) {
    __shared__ double sh[kThreads];
    const std::uint32_t a = blockIdx.x * kThreads + threadIdx.x;
    double q0 = 0.0, q1 = 0.0, q2 = 0.0, q3 = 0.0;
    if (a < g.nodes) {
        const double H = eddy[a] + advective[a];
        out[a] = H;
        const double area = g.area[a];
        q0 = area * H;
        q1 = area * fabs(H);
        q2 = area * fabs(eddy[a]);
        q3 = area * fabs(advective[a]);
    }
    const double s0 = tree_sum(q0, sh), s1 = tree_sum(q1, sh), s2 = tree_sum(q2, sh), s3 = tree_sum(q3, sh);
    if (threadIdx.x == 0) {
        partial[blockIdx.x * kQ + 0] = s0;
        partial[blockIdx.x * kQ + 1] = s1;
        partial[blockIdx.x * kQ + 2] = s2;
        partial[blockIdx.x * kQ + 3] = s3;
    }
}

// ---- the tracer ---------------------------------------------------------------------

struct Stacked {
    std::uint32_t nodes, layers, rows, entries;
    const std::uint32_t* offset;      // stacked CSR
    const std::uint32_t* neighbour;
};

// Each node's upward fluxes W_{l+1/2} (0 for the top) and |final W| (heat_transport.cpp:921-931).
__global__ void k_tracer_vertical(GraphView g, Transport tr, double* __restrict__ vertical,
                                  double* __restrict__ divergence) {
    const std::uint32_t a = blockIdx.x * kThreads + threadIdx.x;
    if (a >= g.nodes) return;
    const std::uint32_t L = tr.layers;
    double w = 0.0;
    for (std::uint32_t l = 0; l < L; ++l) {
        for (std::uint32_t k = g.offset[a]; k < g.offset[a + 1]; ++k) w -= tr.outflow[std::size_t(l) * g.entries + k];
        vertical[std::size_t(a) * L + l] = l + 1 < L ? w : 0.0;
    }
    divergence[a] = fabs(w);
}

// The stacked system's diagonal, off-diagonals and right-hand side (heat_transport.cpp:
// 960-991) and the node-major start c0.
__global__ void k_tracer_assemble(GraphView g, Transport tr, Stacked s, const double* __restrict__ mass, double dt,
                                  double exchange_scale, const double* __restrict__ vertical,
                                  const double* __restrict__ tracer, double* __restrict__ diagonal,
                                  double* __restrict__ off, double* __restrict__ rhs, double* __restrict__ start) {
    const std::uint32_t row = blockIdx.x * kThreads + threadIdx.x;
    if (row >= s.rows) return;
    const std::uint32_t L = tr.layers, a = row / L, l = row % L;
    const double rate = mass[a] / dt;
    double own = rate;
    std::uint32_t at = s.offset[row];
    for (std::uint32_t k = g.offset[a]; k < g.offset[a + 1]; ++k, ++at) {
        const double flow = tr.outflow[std::size_t(l) * g.entries + k];
        const double eddy = tr.conductance[k] * exchange_scale;
        own += std_max(flow, 0.0) + eddy;
        off[at] = -std_max(-flow, 0.0) - eddy;
    }
    const double below = l > 0 ? vertical[std::size_t(a) * L + l - 1] : 0.0;
    const double above = vertical[row];
    if (l > 0) {
        own += std_max(-below, 0.0);
        off[at++] = -std_max(below, 0.0);
    }
    if (l + 1 < L) {
        own += std_max(above, 0.0);
        off[at++] = -std_max(-above, 0.0);
    }
    diagonal[row] = own;
    const double c0 = tracer[std::size_t(l) * g.nodes + a];
    rhs[row] = rate * c0;
    start[row] = c0;
}

// residual = rhs - applied
__global__ void k_sub(std::uint32_t n, const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out) {
    const std::uint32_t i = blockIdx.x * kThreads + threadIdx.x;
    if (i < n) out[i] = a[i] - b[i];
}
// solved = max(0, c0 + delta)
__global__ void k_tracer_solved(std::uint32_t n, const double* __restrict__ start, const double* __restrict__ delta,
                                double* __restrict__ solved) {
    const std::uint32_t i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= n) return;
    solved[i] = std_max(0.0, start[i] + delta[i]);
}
// block partials of sum (rhs - applied)^2 and sum rhs^2
__global__ void __launch_bounds__(kThreads) k_tracer_norms(std::uint32_t n, const double* __restrict__ rhs,
                                                           const double* __restrict__ applied,
                                                           double* __restrict__ partial) {
    __shared__ double sh[kThreads];
    const std::uint32_t i = blockIdx.x * kThreads + threadIdx.x;
    double d = 0.0, r = 0.0;
    if (i < n) {
        d = (rhs[i] - applied[i]) * (rhs[i] - applied[i]);
        r = rhs[i] * rhs[i];
    }
    const double s0 = tree_sum(d, sh), s1 = tree_sum(r, sh);
    if (threadIdx.x == 0) {
        partial[blockIdx.x * kQ + 0] = s0;
        partial[blockIdx.x * kQ + 1] = s1;
    }
}

// The flux form of the solution (heat_transport.cpp:1042-1078), per row in the
// reference's accumulation order: faces from lower nodes (ascending), the vertical flux
// from below, the row's own faces to higher nodes (CSR order), the vertical flux up.
// Then c' = c + dt change / M, clipped at 0 (the mass added is summed in partials).
__global__ void __launch_bounds__(kThreads) k_tracer_flux_form(GraphView g, Transport tr, const double* __restrict__ mass,
                                                               double dt, double exchange_scale,
                                                               const std::uint32_t* __restrict__ face_order,
                                                               const std::uint32_t* __restrict__ lower_count,
                                                               const std::uint32_t* __restrict__ reverse,
                                                               const double* __restrict__ vertical,
                                                               const double* __restrict__ solved,
                                                               const double* __restrict__ tracer,
                                                               double* __restrict__ out, double* __restrict__ partial) {
    __shared__ double sh[kThreads];
    const std::uint32_t L = tr.layers;
    const std::uint32_t row = blockIdx.x * kThreads + threadIdx.x;
    double clipped = 0.0;
    if (row < g.nodes * L) {
        const std::uint32_t a = row / L, l = row % L;
        const std::uint32_t first = g.offset[a], split = first + lower_count[a], last = g.offset[a + 1];
        double change = 0.0;
        for (std::uint32_t idx = first; idx < split; ++idx) {   // faces b -> a, b < a
            const std::uint32_t k = face_order[idx];
            const std::uint32_t b = g.neighbour[k], kb = reverse[k];
            const std::uint32_t donor = b * L + l;
            const double flow = tr.outflow[std::size_t(l) * g.entries + kb];
            const double eddy = tr.conductance[kb] * exchange_scale;
            const double flux = (flow > 0.0 ? flow * solved[donor] : flow * solved[row]) +
                                eddy * (solved[donor] - solved[row]);
            change += flux;
        }
        if (l > 0) {
            const double w = vertical[row - 1];
            change += w > 0.0 ? w * solved[row - 1] : w * solved[row];
        }
        for (std::uint32_t idx = split; idx < last; ++idx) {    // faces a -> b, b > a
            const std::uint32_t k = face_order[idx];
            const std::uint32_t other = g.neighbour[k] * L + l;
            const double flow = tr.outflow[std::size_t(l) * g.entries + k];
            const double eddy = tr.conductance[k] * exchange_scale;
            const double flux = (flow > 0.0 ? flow * solved[row] : flow * solved[other]) +
                                eddy * (solved[row] - solved[other]);
            change -= flux;
        }
        if (l + 1 < L) {
            const double w = vertical[row];
            change -= w > 0.0 ? w * solved[row] : w * solved[row + 1];
        }
        const std::size_t at = std::size_t(l) * g.nodes + a;
        double value = tracer[at] + dt * change / mass[a];
        if (value < 0.0) {
            clipped = -(value * mass[a]);
            value = 0.0;
        }
        out[at] = value;
    }
    const double s = tree_sum(clipped, sh);
    if (threadIdx.x == 0) partial[blockIdx.x * kQ] = s;
}

}  // namespace

// ---- per-planet structures ------------------------------------------------------------

struct NonsymContext {
    DeviceStore store;
    GraphView graph{};
    Ell graph_ell{};
    std::uint32_t* face_order = nullptr;
    std::uint32_t* lower_count = nullptr;
    std::uint32_t* reverse = nullptr;
    std::unique_ptr<DeviceIlu> graph_ilu;
    struct StackedSystem {
        DeviceStore store;
        Stacked view{};
        Ell ell{};
        std::unique_ptr<DeviceIlu> ilu;
    };
    std::map<std::uint32_t, std::unique_ptr<StackedSystem>> stacked;
};

namespace {

// The ELL shape of a CSR pattern (columns slot-major, degrees), in `store`.
Ell ell_of(DeviceStore& store, const std::vector<std::uint32_t>& offset, const std::vector<std::uint32_t>& neighbour) {
    Ell e{};
    e.rows = static_cast<std::uint32_t>(offset.size() - 1);
    for (std::uint32_t r = 0; r < e.rows; ++r) e.width = std::max(e.width, offset[r + 1] - offset[r]);
    if (e.width > 255) throw std::logic_error("non-symmetric solve: a row with more than 255 couplings");
    std::vector<std::uint8_t> degree(e.rows);
    std::vector<std::uint32_t> col(std::size_t(e.width) * e.rows, 0);
    for (std::uint32_t r = 0; r < e.rows; ++r) {
        degree[r] = static_cast<std::uint8_t>(offset[r + 1] - offset[r]);
        for (std::uint32_t j = 0; j < degree[r]; ++j) col[std::size_t(j) * e.rows + r] = neighbour[offset[r] + j];
    }
    e.degree = store.upload(degree);
    e.col = store.upload(col);
    return e;
}

NonsymContext& context(psgb_planet* h) {
    if (h->nonsym) return *h->nonsym;
    upload_planet(*h->planet);
    auto c = std::make_shared<NonsymContext>();
    const TransportGraph& g = h->planet->graph;
    const std::uint32_t n = static_cast<std::uint32_t>(g.size());
    c->graph.nodes = n;
    c->graph.entries = static_cast<std::uint32_t>(g.neighbour.size());
    c->graph.offset = c->store.upload(g.offset);
    c->graph.neighbour = c->store.upload(g.neighbour);
    c->graph.area = h->planet->dev.graph_area;
    std::vector<std::uint32_t> reverse(g.neighbour.size()), order(g.neighbour.size()), lower(n);
    for (std::uint32_t a = 0; a < n; ++a) {
        std::vector<std::pair<std::uint32_t, std::uint32_t>> below;
        std::vector<std::uint32_t> above;
        for (std::uint32_t k = g.offset[a]; k < g.offset[a + 1]; ++k) {
            const std::uint32_t b = g.neighbour[k];
            bool found = false;
            for (std::uint32_t q = g.offset[b]; q < g.offset[b + 1]; ++q) {
                if (g.neighbour[q] == a) {
                    reverse[k] = q;
                    found = true;
                }
            }
            if (!found) throw std::logic_error("transport graph is not symmetric");
            if (b < a) below.emplace_back(b, k);
            else above.push_back(k);
        }
        std::sort(below.begin(), below.end());
        std::uint32_t at = g.offset[a];
        for (const auto& [b, k] : below) order[at++] = k;
        for (std::uint32_t k : above) order[at++] = k;
        lower[a] = static_cast<std::uint32_t>(below.size());
    }
    c->reverse = c->store.upload(reverse);
    c->face_order = c->store.upload(order);
    c->lower_count = c->store.upload(lower);
    c->graph_ilu = std::make_unique<DeviceIlu>(ilu_pattern(g.offset, g.neighbour, fixed_blocks(n, 1)));
    c->graph_ell = ell_of(c->store, g.offset, g.neighbour);
    h->nonsym = c;
    return *c;
}

NonsymContext::StackedSystem& stacked_system(psgb_planet* h, std::uint32_t layers) {
    NonsymContext& c = context(h);
    auto it = c.stacked.find(layers);
    if (it != c.stacked.end()) return *it->second;
    const TransportGraph& g = h->planet->graph;
    const std::uint32_t n = static_cast<std::uint32_t>(g.size());
    // Node-major rows a L + l: the graph row's entries in this layer, then the layer below
    // and the one above (heat_transport.cpp:940-957).
    std::vector<std::uint32_t> offset{0}, neighbour;
    for (std::uint32_t a = 0; a < n; ++a) {
        for (std::uint32_t l = 0; l < layers; ++l) {
            const std::uint32_t row = a * layers + l;
            for (std::uint32_t k = g.offset[a]; k < g.offset[a + 1]; ++k) neighbour.push_back(g.neighbour[k] * layers + l);
            if (l > 0) neighbour.push_back(row - 1);
            if (l + 1 < layers) neighbour.push_back(row + 1);
            offset.push_back(static_cast<std::uint32_t>(neighbour.size()));
        }
    }
    auto s = std::make_unique<NonsymContext::StackedSystem>();
    s->view.nodes = n;
    s->view.layers = layers;
    s->view.rows = n * layers;
    s->view.entries = static_cast<std::uint32_t>(neighbour.size());
    s->view.offset = s->store.upload(offset);
    s->view.neighbour = s->store.upload(neighbour);
    s->ilu = std::make_unique<DeviceIlu>(ilu_pattern(offset, neighbour, fixed_blocks(n, layers)));
    s->ell = ell_of(s->store, offset, neighbour);
    auto& ref = *s;
    c.stacked.emplace(layers, std::move(s));
    return ref;
}

// Device copies of the caller's transport (when it passes host arrays).
struct TransportIn {
    DeviceStore store;
    Transport view{};
};

void load_transport(TransportIn& t, const psgb_advection_diffusion* in, const GraphView& g, int memory,
                    cudaStream_t st) {
    require(in != nullptr && in->conductance_W_K != nullptr && in->outflow_kg_s != nullptr, "null argument");
    require(in->heat_capacity_J_kg_K > 0.0, "the heat capacity must be positive");
    t.view.layers = in->layers;
    t.view.heat_capacity = in->heat_capacity_J_kg_K;
    const std::size_t E = g.entries;
    if (memory == PSGB_MEMORY_DEVICE) {
        t.view.conductance = in->conductance_W_K;
        t.view.outflow = in->outflow_kg_s;
        t.view.latent = in->eddy_latent_W_m2;
        return;
    }
    double* c = t.store.alloc<double>(E);
    double* o = t.store.alloc<double>(std::max<std::size_t>(1, std::size_t(in->layers) * E));
    PSGB_CUDA(cudaMemcpyAsync(c, in->conductance_W_K, E * 8, cudaMemcpyHostToDevice, st));
    if (in->layers > 0)
        PSGB_CUDA(cudaMemcpyAsync(o, in->outflow_kg_s, std::size_t(in->layers) * E * 8, cudaMemcpyHostToDevice, st));
    t.view.conductance = c;
    t.view.outflow = o;
    t.view.latent = nullptr;
    if (in->eddy_latent_W_m2 != nullptr) {
        double* e = t.store.alloc<double>(g.nodes);
        PSGB_CUDA(cudaMemcpyAsync(e, in->eddy_latent_W_m2, std::size_t(g.nodes) * 8, cudaMemcpyHostToDevice, st));
        t.view.latent = e;
    }
}

const double* input(DeviceStore& store, const double* p, std::size_t n, int memory, cudaStream_t st) {
    if (p == nullptr || memory == PSGB_MEMORY_DEVICE) return p;
    double* d = store.alloc<double>(n);
    PSGB_CUDA(cudaMemcpyAsync(d, p, n * 8, cudaMemcpyHostToDevice, st));
    return d;
}

void output(double* dst, const double* src, std::size_t n, int memory, cudaStream_t st) {
    PSGB_CUDA(cudaMemcpyAsync(dst, src, n * 8,
                              memory == PSGB_MEMORY_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
}

void require_memory(int memory) {
    require(memory == PSGB_MEMORY_HOST || memory == PSGB_MEMORY_DEVICE,
            "memory must be PSGB_MEMORY_HOST or PSGB_MEMORY_DEVICE");
}

}  // namespace
}  // namespace psgb

using psgb::capi::guarded;

struct psgb_incomplete_lu {
    psgb::DeviceStore store;
    std::unique_ptr<psgb::DeviceIlu> ilu;
};

extern "C" {

int psgb_incomplete_lu_create(uint32_t rows, const uint32_t* offset, const uint32_t* neighbour, const double* diagonal,
                              const double* off, const uint32_t* block_start, uint32_t blocks, double diagonal_scale,
                              psgb_incomplete_lu** out) {
    return guarded([&] {
        psgb::require(out != nullptr && offset != nullptr && diagonal != nullptr && block_start != nullptr &&
                          (offset[rows] == 0 || (neighbour != nullptr && off != nullptr)),
                      "null argument");
        *out = nullptr;
        std::vector<std::uint32_t> o(offset, offset + rows + 1), nb(neighbour, neighbour + offset[rows]),
            bs(block_start, block_start + blocks + 1);
        auto h = std::make_unique<psgb_incomplete_lu>();
        h->ilu = std::make_unique<psgb::DeviceIlu>(psgb::ilu_pattern(o, nb, bs));
        double* d = h->store.upload(std::vector<double>(diagonal, diagonal + rows));
        double* f = h->store.upload(std::vector<double>(off, off + offset[rows]));
        h->ilu->factor(d, f, diagonal_scale, nullptr);
        *out = h.release();
        return PSGB_OK;
    });
}

int psgb_incomplete_lu_solve(psgb_incomplete_lu* h, double* x, int memory, void* stream) {
    return guarded([&] {
        psgb::require(h != nullptr && x != nullptr, "null argument");
        psgb::require_memory(memory);
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        const std::size_t n = h->ilu->rows();
        if (memory == PSGB_MEMORY_DEVICE) {
            h->ilu->solve(x, st);
            return PSGB_OK;
        }
        psgb::DeviceStore scratch;
        double* d = scratch.alloc<double>(n);
        PSGB_CUDA(cudaMemcpyAsync(d, x, n * 8, cudaMemcpyHostToDevice, st));
        h->ilu->solve(d, st);
        PSGB_CUDA(cudaMemcpyAsync(x, d, n * 8, cudaMemcpyDeviceToHost, st));
        PSGB_CUDA(cudaStreamSynchronize(st));
        return PSGB_OK;
    });
}

void psgb_incomplete_lu_destroy(psgb_incomplete_lu* h) { delete h; }

int psgb_advection_diffusion_source(psgb_planet* planet, const psgb_advection_diffusion* transport,
                                    const double* mean_K, const double* energy_J_kg, double* eddy_W_m2,
                                    double* advective_W_m2, int memory, void* stream) {
    return guarded([&] {
        psgb::require(planet != nullptr && transport != nullptr && mean_K != nullptr && eddy_W_m2 != nullptr &&
                          advective_W_m2 != nullptr,
                      "null argument");
        psgb::require(energy_J_kg != nullptr || transport->layers == 0, "null argument");
        psgb::require_memory(memory);
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        psgb::NonsymContext& c = psgb::context(planet);
        const psgb::GraphView& g = c.graph;
        psgb::TransportIn tr;
        psgb::load_transport(tr, transport, g, memory, st);
        psgb::DeviceStore scratch;
        const double* m = psgb::input(scratch, mean_K, g.nodes, memory, st);
        const double* e = psgb::input(scratch, energy_J_kg, std::size_t(transport->layers) * g.nodes, memory, st);
        double* eo = memory == PSGB_MEMORY_DEVICE ? eddy_W_m2 : scratch.alloc<double>(g.nodes);
        double* ao = memory == PSGB_MEMORY_DEVICE ? advective_W_m2 : scratch.alloc<double>(g.nodes);
        psgb::k_advection_source<<<psgb::blocks_of(g.nodes), psgb::kThreads, 0, st>>>(g, tr.view, m, e, eo, ao);
        PSGB_CHECK_LAUNCH();
        if (memory == PSGB_MEMORY_HOST) {
            psgb::output(eddy_W_m2, eo, g.nodes, memory, st);
            psgb::output(advective_W_m2, ao, g.nodes, memory, st);
        }
        PSGB_CUDA(cudaStreamSynchronize(st));
        return PSGB_OK;
    });
}

int psgb_solve_implicit_tracer(psgb_planet* planet, const psgb_advection_diffusion* transport,
                               const double* layer_mass_kg, const double* tracer, double dt_s,
                               double relative_tolerance, int max_iterations, double* tracer_out,
                               psgb_tracer_result* result, int memory, void* stream) {
    return guarded([&] {
        psgb::require(planet != nullptr && transport != nullptr && layer_mass_kg != nullptr && tracer != nullptr &&
                          tracer_out != nullptr,
                      "null argument");
        psgb::require_memory(memory);
        psgb::require(transport->layers > 0 && dt_s > 0.0, "tracer transport inputs do not match the graph");
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        psgb::NonsymContext& c = psgb::context(planet);
        const psgb::GraphView& g = c.graph;
        const std::uint32_t L = transport->layers;
        psgb::NonsymContext::StackedSystem& S = psgb::stacked_system(planet, L);
        psgb::TransportIn tr;
        psgb::load_transport(tr, transport, g, memory, st);
        psgb::DeviceStore w;
        const double* mass = psgb::input(w, layer_mass_kg, g.nodes, memory, st);
        const double* c0 = psgb::input(w, tracer, std::size_t(L) * g.nodes, memory, st);
        const std::size_t rows = S.view.rows;
        const std::uint32_t urows = static_cast<std::uint32_t>(rows);
        double* vertical = w.alloc<double>(rows);
        double* divergence = w.alloc<double>(g.nodes);
        double* diagonal = w.alloc<double>(rows);
        double* off = w.alloc<double>(S.view.entries);
        double* rhs = w.alloc<double>(rows);
        double* start = w.alloc<double>(rows);
        double* applied = w.alloc<double>(rows);
        double* residual = w.alloc<double>(rows);
        double* delta = w.alloc<double>(rows);
        double* solved = w.alloc<double>(rows);
        double* out = memory == PSGB_MEMORY_DEVICE ? tracer_out : w.alloc<double>(rows);
        const double exchange_scale = 1.0 / (transport->heat_capacity_J_kg_K * static_cast<double>(L));
        const unsigned gn = psgb::blocks_of(g.nodes), gr = psgb::blocks_of(rows);
        psgb::k_tracer_vertical<<<gn, psgb::kThreads, 0, st>>>(g, tr.view, vertical, divergence);
        PSGB_CHECK_LAUNCH();
        psgb::k_tracer_assemble<<<gr, psgb::kThreads, 0, st>>>(g, tr.view, S.view, mass, dt_s, exchange_scale, vertical,
                                                              c0, diagonal, off, rhs, start);
        PSGB_CHECK_LAUNCH();
        S.ilu->factor(diagonal, off, 1.0, st);
        double* off_ell = w.alloc<double>(std::size_t(S.ell.width) * rows);
        psgb::k_csr_to_ell<<<gr, psgb::kThreads, 0, st>>>(S.ell, S.view.offset, off, off_ell);
        PSGB_CHECK_LAUNCH();
        const psgb::Op apply = [&](const double* x, double* y) {
            psgb::k_ell_apply<<<gr, psgb::kThreads, 0, st>>>(S.ell, off_ell, diagonal, x, y);
            PSGB_CHECK_LAUNCH();
        };
        const psgb::Op precondition = [&](const double* x, double* y) {
            psgb::k_copy<<<gr, psgb::kThreads, 0, st>>>(urows, x, y);
            PSGB_CHECK_LAUNCH();
            S.ilu->solve(y, st);
        };
        // A delta = b - A c0, from delta = 0.
        apply(start, applied);
        psgb::k_sub<<<gr, psgb::kThreads, 0, st>>>(urows, rhs, applied, residual);
        PSGB_CHECK_LAUNCH();
        psgb::Scalars sc(w, rows);
        const psgb::BicgWork work(w, rows);
        psgb_tracer_result r{};
        r.iterations = psgb::bicgstab(rows, apply, precondition, residual, delta, relative_tolerance, max_iterations,
                                      work, sc, st);
        psgb::k_tracer_solved<<<gr, psgb::kThreads, 0, st>>>(urows, start, delta, solved);
        PSGB_CHECK_LAUNCH();
        apply(solved, applied);
        psgb::k_tracer_norms<<<gr, psgb::kThreads, 0, st>>>(urows, rhs, applied, sc.partial());
        PSGB_CHECK_LAUNCH();
        const auto [residual_norm, rhs_norm] = sc.read(2, 0u, st);
        r.relative_residual = rhs_norm > 0.0 ? std::sqrt(residual_norm / rhs_norm) : 0.0;
        std::vector<double> div(g.nodes);   // the largest column divergence, below
        PSGB_CUDA(cudaMemcpyAsync(div.data(), divergence, g.nodes * 8, cudaMemcpyDeviceToHost, st));
        psgb::k_tracer_flux_form<<<gr, psgb::kThreads, 0, st>>>(g, tr.view, mass, dt_s, exchange_scale, c.face_order,
                                                               c.lower_count, c.reverse, vertical, solved, c0, out,
                                                               sc.partial());
        PSGB_CHECK_LAUNCH();
        r.clipped_kg = sc.read(1, 0u, st).first;
        for (double d : div) r.column_divergence_kg_s = std::max(r.column_divergence_kg_s, d);
        if (memory == PSGB_MEMORY_HOST) psgb::output(tracer_out, out, rows, memory, st);
        PSGB_CUDA(cudaStreamSynchronize(st));
        if (result != nullptr) *result = r;
        return PSGB_OK;
    });
}

int psgb_solve_implicit_advection_diffusion(psgb_planet* planet, const psgb_advection_diffusion* transport,
                                            const double* source_floor_W_m2, const double* initial_source_W_m2,
                                            psgb_advection_response host_response,
                                            psgb_device_advection_response device_response, void* user,
                                            const psgb_transport_settings* settings_in, double* source_out_W_m2,
                                            double* mean_out_K, double* energy_out_J_kg,
                                            psgb_advection_result* result, int memory, void* stream) {
    return guarded([&] {
        psgb::require(planet != nullptr && transport != nullptr && source_floor_W_m2 != nullptr &&
                          source_out_W_m2 != nullptr && (host_response != nullptr) != (device_response != nullptr),
                      "null argument (give exactly one of the host and device responses)");
        psgb::require_memory(memory);
        psgb_transport_settings settings;
        psgb_transport_settings_default(&settings);
        if (settings_in != nullptr) settings = *settings_in;
        psgb::require(settings.max_newton_iterations >= 0 && settings.max_line_search_halvings >= 0 &&
                          settings.max_non_monotone_steps >= 0 && settings.max_cg_iterations > 0,
                      "iteration limits must not be negative");
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        psgb::NonsymContext& c = psgb::context(planet);
        const psgb::GraphView& g = c.graph;
        const std::uint32_t n = g.nodes, L = transport->layers;
        const std::size_t nl = std::size_t(L) * n;
        psgb::TransportIn tr;
        psgb::load_transport(tr, transport, g, memory, st);
        {   // eddy conductances must be finite and non-negative (heat_transport.cpp:1094-1098)
            std::vector<double> G(g.entries);
            PSGB_CUDA(cudaMemcpyAsync(G.data(), tr.view.conductance, G.size() * 8, cudaMemcpyDeviceToHost, st));
            PSGB_CUDA(cudaStreamSynchronize(st));
            for (double v : G)
                psgb::require(v >= 0.0 && std::isfinite(v), "eddy conductances must be finite and non-negative");
        }
        psgb::DeviceStore w;
        const double* floor = psgb::input(w, source_floor_W_m2, n, memory, st);
        const double* initial = psgb::input(w, initial_source_W_m2, n, memory, st);
        struct Iterate {
            double *source, *mean, *slope, *energy, *energy_slope, *residual;
            double merit, largest;
        };
        auto make = [&] {
            return Iterate{w.alloc<double>(n), w.alloc<double>(n), w.alloc<double>(n), w.alloc<double>(std::max<std::size_t>(1, nl)),
                           w.alloc<double>(std::max<std::size_t>(1, nl)), w.alloc<double>(n), 0.0, 0.0};
        };
        Iterate current = make(), trial = make();
        double* eddy = w.alloc<double>(n);
        double* advective = w.alloc<double>(n);
        double* diagonal = w.alloc<double>(n);
        double* off = w.alloc<double>(g.entries);
        double* sym_diagonal = w.alloc<double>(n);
        double* sym_off = w.alloc<double>(g.entries);
        double* rhs = w.alloc<double>(n);
        double* delta = w.alloc<double>(n);
        double* scaled = w.alloc<double>(n);
        double* leftover = w.alloc<double>(n);
        psgb::Scalars sc(w, n);
        const psgb::BicgWork work(w, n);
        const unsigned gn = psgb::blocks_of(n);
        // host copies for a host response
        psgb::PinnedDoubles host;
        if (host_response != nullptr) host.reset(3 * std::size_t(n) + 2 * nl + 1);
        auto respond = [&](Iterate& at) {
            if (device_response != nullptr) {
                if (device_response(user, n, L, at.source, at.mean, at.slope, at.energy, at.energy_slope, st) != 0)
                    throw std::runtime_error("the advection response callback failed");
                return;
            }
            double* hs = host.data();
            double *hm = hs + n, *hsl = hm + n, *he = hsl + n, *hes = he + nl;
            PSGB_CUDA(cudaMemcpyAsync(hs, at.source, std::size_t(n) * 8, cudaMemcpyDeviceToHost, st));
            PSGB_CUDA(cudaStreamSynchronize(st));
            if (host_response(user, n, L, hs, hm, hsl, he, hes) != 0)
                throw std::runtime_error("the advection response callback failed");
            PSGB_CUDA(cudaMemcpyAsync(at.mean, hm, std::size_t(n) * 8, cudaMemcpyHostToDevice, st));
            PSGB_CUDA(cudaMemcpyAsync(at.slope, hsl, std::size_t(n) * 8, cudaMemcpyHostToDevice, st));
            if (nl > 0) {
                PSGB_CUDA(cudaMemcpyAsync(at.energy, he, nl * 8, cudaMemcpyHostToDevice, st));
                PSGB_CUDA(cudaMemcpyAsync(at.energy_slope, hes, nl * 8, cudaMemcpyHostToDevice, st));
            }
        };
        // F(h) = h - H(theta(h), s(h)) and the merit sum A F^2 (heat_transport.cpp:1111-1133).
        auto evaluate = [&](Iterate& at) {
            respond(at);
            psgb::k_advection_source<<<gn, psgb::kThreads, 0, st>>>(g, tr.view, at.mean, at.energy, eddy, advective);
            PSGB_CHECK_LAUNCH();
            psgb::k_advection_residual<<<gn, psgb::kThreads, 0, st>>>(g, at.source, eddy, advective, at.residual,
                                                                     sc.partial());
            PSGB_CHECK_LAUNCH();
            const auto [merit, largest] = sc.read(2, 0x2u, st);
            at.merit = merit;
            at.largest = largest;
        };
        psgb::k_advection_start<<<gn, psgb::kThreads, 0, st>>>(n, initial, floor, current.source);
        PSGB_CHECK_LAUNCH();
        evaluate(current);
        psgb_advection_result out{};
        int non_monotone = 0;
        double* off_ell = w.alloc<double>(std::size_t(c.graph_ell.width) * n);
        const psgb::Op apply = [&](const double* x, double* y) {
            psgb::k_ell_apply<<<gn, psgb::kThreads, 0, st>>>(c.graph_ell, off_ell, diagonal, x, y);
            PSGB_CHECK_LAUNCH();
        };
        // The V-cycle of A theta'^-1 + K on A x, divided by theta', then the block ILU of J
        // on what is left (heat_transport.cpp:1233-1249).
        const psgb::Op precondition = [&](const double* x, double* y) {
            psgb::k_scale_area<<<gn, psgb::kThreads, 0, st>>>(n, g.area, x, scaled);
            PSGB_CHECK_LAUNCH();
            if (psgb_multigrid_precondition(planet, PSGB_DTYPE_F64, scaled, y, PSGB_MEMORY_DEVICE, st) != PSGB_OK)
                throw std::runtime_error(psgb_last_error());
            psgb::k_unscale_slope<<<gn, psgb::kThreads, 0, st>>>(n, current.slope, y);
            PSGB_CHECK_LAUNCH();
            apply(y, leftover);
            psgb::k_leftover<<<gn, psgb::kThreads, 0, st>>>(n, x, leftover);
            PSGB_CHECK_LAUNCH();
            c.graph_ilu->solve(leftover, st);
            psgb::k_add<<<gn, psgb::kThreads, 0, st>>>(n, leftover, y);
            PSGB_CHECK_LAUNCH();
        };
        for (int iteration = 0; iteration < settings.max_newton_iterations; ++iteration) {
            if (current.largest <= settings.newton_tolerance_W_m2) break;
            psgb::k_advection_jacobian<<<gn, psgb::kThreads, 0, st>>>(g, tr.view, current.slope, current.energy_slope,
                                                                     current.residual, diagonal, off, rhs, sym_diagonal,
                                                                     sym_off);
            PSGB_CHECK_LAUNCH();
            c.graph_ilu->factor(diagonal, off, 1.0, st);
            psgb::k_csr_to_ell<<<gn, psgb::kThreads, 0, st>>>(c.graph_ell, g.offset, off, off_ell);
            PSGB_CHECK_LAUNCH();
            if (psgb_multigrid_set_matrix(planet, sym_diagonal, sym_off, PSGB_MEMORY_DEVICE, st) != PSGB_OK)
                throw std::runtime_error(psgb_last_error());
            out.linear_iterations += psgb::bicgstab(n, apply, precondition, rhs, delta, settings.cg_relative_tolerance,
                                                    settings.max_cg_iterations, work, sc, st);
            // Backtracking on the merit (heat_transport.cpp:1255-1292).
            double step = 1.0;
            bool accepted = false;
            for (int halving = 0;; ++halving) {
                psgb::k_advection_trial<<<gn, psgb::kThreads, 0, st>>>(n, current.source, delta, step, floor,
                                                                      trial.source);
                PSGB_CHECK_LAUNCH();
                evaluate(trial);
                if (trial.merit < current.merit) {
                    accepted = true;
                    break;
                }
                if (halving == settings.max_line_search_halvings) {
                    if (current.largest > settings.rounding_floor_W_m2 &&
                        non_monotone < settings.max_non_monotone_steps) {
                        ++non_monotone;
                        psgb::k_advection_trial<<<gn, psgb::kThreads, 0, st>>>(n, current.source, delta, 1.0, floor,
                                                                              trial.source);
                        PSGB_CHECK_LAUNCH();
                        evaluate(trial);
                        accepted = std::isfinite(trial.merit) &&
                                   trial.merit <= settings.max_non_monotone_growth * current.merit;
                    }
                    break;
                }
                step *= 0.5;
            }
            if (!accepted) break;
            std::swap(current, trial);
            ++out.newton_iterations;
        }
        // The transport applied: the conservative source of the last iterate's theta and s.
        psgb::k_advection_source<<<gn, psgb::kThreads, 0, st>>>(g, tr.view, current.mean, current.energy, eddy,
                                                               advective);
        PSGB_CHECK_LAUNCH();
        double* H = memory == PSGB_MEMORY_DEVICE ? source_out_W_m2 : w.alloc<double>(n);
        psgb::k_advection_final<<<gn, psgb::kThreads, 0, st>>>(g, eddy, advective, H, sc.partial());
        PSGB_CHECK_LAUNCH();
        psgb::k_finish<<<1, psgb::kThreads, 0, st>>>(sc.blocks(), 4, 0u, sc.partial(), scaled);
        PSGB_CHECK_LAUNCH();
        double sums[4];
        PSGB_CUDA(cudaMemcpyAsync(sums, scaled, sizeof(sums), cudaMemcpyDeviceToHost, st));
        if (memory == PSGB_MEMORY_HOST) psgb::output(source_out_W_m2, H, n, memory, st);
        if (mean_out_K != nullptr) psgb::output(mean_out_K, current.mean, n, memory, st);
        if (energy_out_J_kg != nullptr && nl > 0) psgb::output(energy_out_J_kg, current.energy, nl, memory, st);
        PSGB_CUDA(cudaStreamSynchronize(st));
        out.consistency_residual_W_m2 = current.largest;
        out.sum_W = sums[0];
        out.absolute_sum_W = sums[1];
        out.eddy_absolute_sum_W = sums[2];
        out.advective_absolute_sum_W = sums[3];
        if (result != nullptr) *result = out;
        return PSGB_OK;
    });
}

}  // extern "C"
