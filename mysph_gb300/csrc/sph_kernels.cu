// sph_kernels.cu — the per-step kernels of the GB300 SPH hot path.
//
//   keys        cell key of every real particle (+ per-cell counts)
//   permute     gather the state into cell order; leap-frog half kick
//               (timeIntegration.f90:137-170) fused in
//   pass A      density rate, divergence, velocity gradient -> strain /
//               rotation rate; EOS, viscous entropy, Jaumann stress rate and
//               stress in the epilogue (density.f90:83-107,
//               divergence.f90:6-29, internalForce.f90:44-189)
//   pass B      momentum and energy: internal force, artificial viscosity,
//               external (gravity, wall repulsion, penalty, contact) and
//               artificial-stress pair terms, assembled with the fixed
//               boundary (internalForce.f90:194-334, artificialViscosity.f90,
//               externalForce.f90, artificialTerm.f90, singleStep.f90:139-144,
//               boundaryCondition.f90:32-45)
//   update      leap-frog full update, radial return, Courant statistics
//               (timeIntegration.f90:178-252, courantNumber.f90:7-31)
//
// Neighbour search (replaces BGGS, asymmetricSearch.f90:160-257): every
// target walks the 3^(dim-1) rows of cells around its cell in the real and
// in the wall grid.  A warp first filters candidates with FP32 positions and
// a guard band (candidates inside the band get the reference's exact FP64
// test: dx = x_i - x_j, dr = sum dx^2 without FMA, r = sqrt(dr) < scale_k h_i)
// and appends accepted indices to a per-lane list in shared memory; the
// FP64 pair physics then runs over the lists with all lanes busy.  No pair
// list ever reaches global memory.
#include <algorithm>
#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

#include "sph_device.cuh"
#include "sph_kernels.cuh"

namespace sph {
namespace {

constexpr int TPB = 128;          // threads per block of the pair passes
constexpr int MAX_TILE_TPB = 128; // largest block of the tiled (mixed) passes
// Blocks per SM the mixed passes are compiled for (a register budget):
// measured on the 256-system 2-D ensemble against the compiler's own choice,
// pass A 1.158 -> 1.085 ms at 6, pass B 1.770 -> 1.599 ms at 5 (8 spilled and
// lost).  The 3-D forms are compiled for 4 blocks of 128 threads (at most 128
// registers): at 5, pass A took 1.49 ms against 1.40, and with no minimum
// (up to 255 registers) pass B took 2.34 ms against 1.99.
constexpr int MIXED_A_MINB_2D = 6;
constexpr int MIXED_B_MINB_2D = 5;
constexpr int WARPS = TPB / 32;
// Per warp in shared memory: K accepted neighbour indices per lane, then a
// tile of 32 staged candidate positions (float4).
// The tiled walk (mixed passes) flushes when a list could overflow on the
// next tile of 32, so it gets longer lists by default in 3-D (88: 47 KB per
// block of 4 warps, under the default 48 KB of dynamic shared memory); its
// list length and block size are context options (the autotuner's knobs).
// K list entries per lane, then the staging tile of 32 float4 (and a second
// one for the candidates' velocities when the walk splits by approach)
// Per-warp words of the mixed kernels, whose list length K is a launch
// option: the list and the position tile.  (Their pass B does not split its
// lists by approach: in FP32 the split cost more than the AV branch saves,
// and it would tie the summation order to K.)
constexpr int tiled_slot(int k) { return k * 32 + 32 * 4; }
template <int DIM, bool TILED = false, bool SPLIT = false> struct ListLen {
    static constexpr int K = DIM == 2 ? 64 : (TILED ? 88 : 72);
    static constexpr int SLOT = K * 32 + 32 * 4 * (SPLIT ? 2 : 1);  // in uint32 words
};

__device__ __forceinline__ double cmp(const double4& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }
__device__ __forceinline__ void setc(double4& v, int a, double x) {
    if (a == 0) v.x = x; else if (a == 1) v.y = x; else v.z = x;
}

// ---------------------------------------------------------------------------
// target description and the neighbour walk
// ---------------------------------------------------------------------------
template <int DIM>
__device__ __forceinline__ KConstF make_kconst_f(int skf, double h) {
    const KConst k = make_kconst<DIM>(skf, h);
    KConstF f;
    f.hinv = (float)k.hinv;
    f.factor = (float)k.factor;
    f.A1 = (float)k.A1;
    f.A2 = (float)k.A2;
    f.A3 = (float)k.A3;
    return f;
}

// The reference constants of target i's system when its h has the
// reference's bits and the kernel is theirs (an integer compare, no FP64
// instruction); else null, and the caller computes its own.
__device__ __forceinline__ const KRef* kref_for(const Dev& d, int i, int skf, double h) {
    const KRef* r = d.kref + d.pinst[i];
    return (__double_as_longlong(h) == __double_as_longlong(r->h) && r->skf == skf) ? r : nullptr;
}
template <int DIM>
__device__ __forceinline__ KConst kconst_of(const Dev& d, int i, int skf, double h) {
    const KRef* r = kref_for(d, i, skf, h);
    return r ? r->k : make_kconst<DIM>(skf, h);
}
template <int DIM>
__device__ __forceinline__ KConstF kconst_f_of(const Dev& d, int i, int skf, double h) {
    const KRef* r = kref_for(d, i, skf, h);
    return r ? r->kf : make_kconst_f<DIM>(skf, h);
}

// Candidate-test bounds of a target with smoothing length h (make_target,
// and kref_kernel for the reference h): the exact test's reach, and the FP32
// r^2 band around it inside which that test decides.
__device__ __forceinline__ void reach_bounds(const Dev& d, const Grid& g, double h, double* reach, float* lo2,
                                             float* hi2) {
    *reach = h * (double)d.scale_k;
    const double r2 = *reach * *reach;
    *lo2 = __double2float_rd(r2 * (1.0 - (double)g.guard));
    *hi2 = __double2float_ru(r2 * (1.0 + (double)g.guard));
}

template <int DIM>
struct Target {
    int i;           // combined (sorted) index
    double x[3];
    float xf[3];
    float lo2, hi2;  // FP32 r^2 thresholds: accept below lo2, exact test up to hi2
    double reach;    // scale_k * h_i (the exact FP64 test)
    bool far;        // target outside the grid domain: FP32 filter not valid
    int cell[3];
    int nc[3];       // cells per axis of the target's instance grid
    int base;        // its first global cell
};

template <int DIM>
__device__ __forceinline__ Target<DIM> make_target(const Dev& d, int i, const double4& xm, double h) {
    Target<DIM> t;
    t.i = i;
    t.x[0] = xm.x; t.x[1] = xm.y; t.x[2] = DIM == 3 ? xm.z : 0.0;
    float4 pf = d.posf[i];
    t.xf[0] = pf.x; t.xf[1] = pf.y; t.xf[2] = pf.z;
    t.far = pf.w != 0.0f;
    const Inst& I = inst_of(d, i);
    if (const KRef* r = kref_for(d, i, d.skf, h)) {
        t.reach = r->reach;
        t.lo2 = r->lo2;
        t.hi2 = r->hi2;
    } else {
        reach_bounds(d, I.grid, h, &t.reach, &t.lo2, &t.hi2);
    }
    // the cell of the current search (the positions have not moved since)
    cell_from_key(I.grid, I.cell_base, d.keys_s[i], t.cell);
    t.nc[0] = I.grid.nc[0]; t.nc[1] = I.grid.nc[1]; t.nc[2] = I.grid.nc[2];
    t.base = I.cell_base;
    return t;
}

// The reference's distance test, operation for operation
// (asymmetricSearch.f90:227-237): no FMA contraction, correctly rounded sqrt.
template <int DIM>
__device__ __forceinline__ bool exact_in_range(const Target<DIM>& t, const double4& xj) {
    double dx0 = __dsub_rn(t.x[0], xj.x);
    double dr = __dmul_rn(dx0, dx0);
    double dx1 = __dsub_rn(t.x[1], xj.y);
    dr = __dadd_rn(dr, __dmul_rn(dx1, dx1));
    if (DIM == 3) {
        double dx2 = __dsub_rn(t.x[2], xj.z);
        dr = __dadd_rn(dr, __dmul_rn(dx2, dx2));
    }
    return __dsqrt_rn(dr) < t.reach;
}

template <int DIM>
__device__ __forceinline__ bool accept(const Dev& d, const Target<DIM>& t, int j, const float4& pj) {
    if (j == t.i) return false;
    float ex = t.xf[0] - pj.x, ey = t.xf[1] - pj.y;
    float d2 = ex * ex + ey * ey;
    if (DIM == 3) { float ez = t.xf[2] - pj.z; d2 += ez * ez; }
    // particles outside the grid domain (posf.w != 0) always take the exact test
    if (!t.far && pj.w == 0.0f) {
        if (d2 < t.lo2) return true;
        if (d2 > t.hi2) return false;
    }
    return exact_in_range<DIM>(t, d.xm[j]);
}

// The FP64 path's candidate test as a policy of walk().
template <int DIM>
struct ExactAccept {
    const Dev& d;
    const Target<DIM>& t;
    __device__ __forceinline__ bool operator()(int j, const float4& pj) const { return accept<DIM>(d, t, j, pj); }
};

// Walk all neighbours of the lane's target and call ph.pair(j) for each
// candidate `acc` accepts.  Every lane of the warp must call it (inactive
// lanes with active=false).  Two forms with the same neighbour order:
//
// walk_lane: each lane steps through its own 3^(dim-1) row ranges one
// candidate per iteration (its FP32 position loaded from L1/L2); a lane's
// list fills at a steady rate, so the pair physics runs on nearly full lists.
// Used by the once-per-search passes (S, K, R) and the neighbour export.
template <int DIM, int K, class Phys, class Acc>
__device__ __forceinline__ void walk_lane(const Dev& d, const Target<DIM>& t, bool active, Phys& ph,
                                          uint32_t* lst, const Acc& acc) {
    constexpr int NR = DIM == 2 ? 3 : 9;
    const int lane = threadIdx.x & 31;
    int r = 0, cur = 0, end = 0;
    bool more = active;
    auto next_range = [&]() {
        while (r < 2 * NR) {
            const int rr = r < NR ? r : r - NR;
            const int cy = t.cell[1] + (DIM == 2 ? rr - 1 : (rr % 3) - 1);
            const int cz = t.cell[2] + (DIM == 2 ? 0 : (rr / 3) - 1);
            const bool wall = r >= NR;
            ++r;
            if (cy < 0 || cy >= t.nc[1] || cz < 0 || cz >= t.nc[2]) continue;
            const int cx0 = max(t.cell[0] - 1, 0), cx1 = min(t.cell[0] + 1, t.nc[0] - 1);
            const int row = t.base + (cz * t.nc[1] + cy) * t.nc[0];
            const int* st = wall ? d.wstart : d.fstart;
            const int b = st[row + cx0], e = st[row + cx1 + 1];
            if (b < e) {
                const int off = wall ? d.wall_off : 0;
                cur = b + off;
                end = e + off;
                return;
            }
        }
        more = false;
    };
    if (more) next_range();
    while (true) {
        int cnt = 0;
        while (__any_sync(SPH_FULL_MASK, more)) {
            if (more) {
                if (acc(cur, d.posf[cur])) { lst[cnt * 32 + lane] = (uint32_t)cur; ++cnt; }
                if (++cur >= end) next_range();
            }
            if (__any_sync(SPH_FULL_MASK, cnt >= K)) break;
        }
        const int mc = warp_max_int(cnt);
        for (int k = 0; k < mc; ++k)
            if (k < cnt) ph.pair((int)lst[k * 32 + lane]);
        if (!__any_sync(SPH_FULL_MASK, more)) break;
    }
}

// walk_tiled: the warp groups its lanes by cell row (targets are in cell
// order, so a warp usually covers one row).  For each group it walks the
// 3^(dim-1) neighbour rows of the real and of the wall grid over the group's
// x-range widened by one cell.  Each range is loaded 32 candidates at a time
// into a shared-memory tile (one coalesced 512-byte load), and every lane of
// the group tests all staged candidates from
// broadcast shared-memory reads into a 32-bit acceptance mask.  Accepted
// indices go to the lane's list; the pair physics runs over the lists with
// all lanes busy whenever a list could overflow on the next tile (more than
// K - 32 entries).  Within a row the accepted neighbours come in increasing
// index order, rows in a fixed order, so the summation order does not
// depend on the warp's other targets.  Used by passes A and B in every
// precision (EXACT in FP64 and DF64): it removes the per-candidate L1/L2
// latency of the per-lane walk.
//
// EXACT: the FP64 path's candidate test instead of the FP32 cut at reach2
// (accept below the guard band, the reference's FP64 distance test inside
// it), so the neighbour sets are those of walk_lane with ExactAccept.
//
// Split (pass B): the accepted neighbours whose FP32 estimate of
// (x_i - x_j).(v_i - v_j) is negative, the approaching pairs that take the
// artificial viscosity, fill the list from the front and the others from the
// back; the pair physics runs over the front part first.  The warp then runs
// the AV branch only while some lane is still in its approaching part,
// instead of on nearly every pair.  The estimate only orders the list: the
// physics decides on the exact sign.
struct NoSplit {
    static constexpr bool on = false;
    float vx = 0.0f, vy = 0.0f, vz = 0.0f;
    __device__ __forceinline__ float4 vel(int) const { return make_float4(0.0f, 0.0f, 0.0f, 0.0f); }
};
struct SplitFP64 {   // candidates' velocities rounded from the FP64 state
    // (d2f: the rounding of the conversion instruction, on the integer pipes,
    // which the FP64 pair passes leave mostly idle, instead of the FP64 pipe,
    // which binds them)
    static constexpr bool on = true;
    const Dev& d;
    float vx, vy, vz;
    __device__ SplitFP64(const Dev& dd, const double4& v) : d(dd), vx(d2f(v.x)), vy(d2f(v.y)), vz(d2f(v.z)) {}
    __device__ __forceinline__ float4 vel(int j) const {
        const double4 v = d.vr[j];
        return make_float4(d2f(v.x), d2f(v.y), d2f(v.z), 0.0f);
    }
};
struct SplitDF {     // the high parts of the double-float velocity mirror
    static constexpr bool on = true;
    const Dev& d;
    float vx, vy, vz;
    __device__ SplitDF(const Dev& dd, int i) : d(dd) {
        const float4 v = d.vd0[i];
        vx = v.x; vy = v.y; vz = v.z;
    }
    __device__ __forceinline__ float4 vel(int j) const { return d.vd0[j]; }
};

// Pair physics with `static constexpr bool early_entry = true` have the walk
// read each list entry one pair ahead, so that the shared-memory read of the
// next index overlaps the current pair.  It pays where the pair loop waits on
// latency (the 3-D mixed pass B, 4 %); the FP64 and double-float passes,
// bound by issue, and the 2-D mixed pass B gain nothing or lose.
template <class T, class = void>
struct EarlyEntry : std::false_type {};
template <class T>
struct EarlyEntry<T, std::void_t<decltype(T::early_entry)>> : std::bool_constant<T::early_entry> {};

// Lanes per target (SPH_OPT_LANES, FP64 passes A and B): a group of L
// consecutive lanes holds the same target and walks its candidates together.
// Each lane tests every L-th staged candidate and the group joins the masks;
// the k-th accepted neighbour of the target's own sequence goes to lane
// k mod L of the group, so each lane's pairs, and the fixed butterfly that
// adds the L partial sums (lane_sum), depend on the target alone.  Every lane
// of the group ends with the same bits.
struct NoShare {
    static constexpr bool on = false;
    __device__ __forceinline__ unsigned take(unsigned m) { return m; }
};
struct LaneShare {
    static constexpr bool on = true;
    int sub, lmask;  // lane within the group, L - 1
    int seen = 0;    // neighbours of the target accepted so far
    // the union of the group's acceptance masks (every lane of the warp calls it)
    __device__ __forceinline__ unsigned join(unsigned m) const {
        for (int o = 1; o <= lmask; o <<= 1) m |= __shfl_xor_sync(SPH_FULL_MASK, m, o);
        return m;
    }
    // this lane's share of the accepted candidates
    __device__ __forceinline__ unsigned take(unsigned m) {
        unsigned sel = 0u;
        int k = seen;
        while (m) {
            const int q = __ffs(m) - 1;
            m &= m - 1u;
            if ((k & lmask) == sub) sel |= 1u << q;
            ++k;
        }
        seen = k;
        return sel;
    }
};
__device__ __forceinline__ double lane_sum(double v, int L) {
    for (int o = 1; o < L; o <<= 1) v += __shfl_xor_sync(SPH_FULL_MASK, v, o);
    return v;
}
__device__ __forceinline__ int lane_sum(int v, int L) {
    for (int o = 1; o < L; o <<= 1) v += __shfl_xor_sync(SPH_FULL_MASK, v, o);
    return v;
}

template <int DIM, int K, class Phys, bool EXACT = false, class Split = NoSplit, class Share = NoShare>
__device__ __forceinline__ void walk_tiled(const Dev& d, const Target<DIM>& t, bool active, Phys& ph,
                                           uint32_t* lst, float4* tile, float reach2,
                                           const Split& sp = Split{}, Share sh = Share{}) {
    constexpr int NR = DIM == 2 ? 3 : 9;
    static_assert(K >= 64, "a tile of 32 candidates needs room for 32 more entries");
    const int lane = threadIdx.x & 31;
    const int my_row = t.base + (t.cell[2] * t.nc[1] + t.cell[1]) * t.nc[0];
    const float x0 = t.xf[0], x1 = t.xf[1], x2 = t.xf[2];
    unsigned pending = __ballot_sync(SPH_FULL_MASK, active);
    int cnt = 0, nb = 0;   // entries at the front and (Split) at the back of the list
    float4* tilev = tile + 32;
    // The mixed passes keep the staged candidates as three arrays (x, y, z),
    // so that one broadcast 64-bit load brings the same coordinate of two
    // candidates and the FP32 distance test runs on pairs of candidates with
    // the packed instructions (FADD2 / FMUL2 / FFMA2); dx is formed as
    // p - x_i, the negative of x_i - p, so each squared distance keeps its
    // rounding.  The exact form (FP64, DF64) stages float4 rows.
    float* tx = reinterpret_cast<float*>(tile);
    float* ty = tx + 32;
    float* tz = tx + 64;
    const float2 nx0 = make_float2(-x0, -x0), nx1 = make_float2(-x1, -x1), nx2 = make_float2(-x2, -x2);
    // run the pair physics over the lists of the lanes that take part: the
    // front part, then the back part in the order it was filled
    auto flush = [&](bool take) {
        const int tot = take ? cnt + nb : 0;
        const int mc = warp_max_int(tot);
        auto entry = [&](int k) { return (int)lst[(k < cnt ? k : K - 1 - (k - cnt)) * 32 + lane]; };
        if constexpr (EarlyEntry<Phys>::value) {
            int jn = tot > 0 ? entry(0) : 0;
            for (int k = 0; k < mc; ++k) {
                const int j = jn;
                if (k + 1 < tot) jn = entry(k + 1);
                if (k < tot) ph.pair(j);
            }
        } else {
            for (int k = 0; k < mc; ++k)
                if (k < tot) ph.pair(entry(k));
        }
        if (take) cnt = nb = 0;
    };
    while (pending) {
        const int leader = __ffs(pending) - 1;
        const int grow = __shfl_sync(SPH_FULL_MASK, my_row, leader);
        const bool mine = active && my_row == grow;
        pending &= ~__ballot_sync(SPH_FULL_MASK, mine);
        const int cy = __shfl_sync(SPH_FULL_MASK, t.cell[1], leader);
        const int cz = __shfl_sync(SPH_FULL_MASK, t.cell[2], leader);
        const int nc0 = __shfl_sync(SPH_FULL_MASK, t.nc[0], leader);
        const int nc1 = __shfl_sync(SPH_FULL_MASK, t.nc[1], leader);
        const int nc2 = __shfl_sync(SPH_FULL_MASK, t.nc[2], leader);
        const int base = __shfl_sync(SPH_FULL_MASK, t.base, leader);
        const int cx0 = max(warp_min_int(mine ? t.cell[0] : 0x7fffffff) - 1, 0);
        const int cx1 = min(warp_max_int(mine ? t.cell[0] : -1) + 1, nc0 - 1);
        for (int r = 0; r < 2 * NR; ++r) {
            const int rr = r < NR ? r : r - NR;
            const int y = cy + (DIM == 2 ? rr - 1 : (rr % 3) - 1);
            const int z = cz + (DIM == 2 ? 0 : (rr / 3) - 1);
            if (y < 0 || y >= nc1 || z < 0 || z >= nc2) continue;
            const bool wall = r >= NR;
            const int row = base + (z * nc1 + y) * nc0;
            const int* st = wall ? d.wstart : d.fstart;
            const int off = wall ? d.wall_off : 0;
            const int b = st[row + cx0] + off, e = st[row + cx1 + 1] + off;
            for (int c0 = b; c0 < e; c0 += 32) {
                const int n = min(32, e - c0);
                if (lane < n) {
                    const float4 p = d.posf[c0 + lane];
                    if constexpr (EXACT) {
                        tile[lane] = p;
                    } else {
                        tx[lane] = p.x;
                        ty[lane] = p.y;
                        tz[lane] = p.z;
                    }
                    if constexpr (Split::on) tilev[lane] = sp.vel(c0 + lane);
                }
                __syncwarp();
                unsigned m = 0u;
                if (mine) {
                    // acceptance mask of the staged candidates (entries past n
                    // hold stale data and are masked off)
                    unsigned maybe = 0u;
                    if constexpr (EXACT) {
                        // the FP64 and DF64 passes are bound by their pair
                        // physics: the plain form keeps registers for it
                        auto test = [&](int q) {
                            const float4 p = tile[q];
                            const float ex = x0 - p.x, ey = x1 - p.y;
                            float d2 = ex * ex + ey * ey;
                            if (DIM == 3) { const float ez = x2 - p.z; d2 += ez * ez; }
                            const bool plain = !t.far && p.w == 0.0f;
                            m |= (plain && d2 < t.lo2 ? 1u : 0u) << q;
                            maybe |= (!plain || (d2 >= t.lo2 && d2 <= t.hi2) ? 1u : 0u) << q;
                        };
                        if constexpr (Share::on) {
                            // each lane of the group tests every L-th candidate;
                            // the group's masks are joined below
                            for (int q = sh.sub; q < 32; q += sh.lmask + 1) test(q);
                        } else {
#pragma unroll
                            for (int q = 0; q < 32; ++q) test(q);
                        }
                    } else {
#pragma unroll
                        for (int q = 0; q < 32; q += 2) {
                            const float2 X = *reinterpret_cast<const float2*>(tx + q);
                            const float2 Y = *reinterpret_cast<const float2*>(ty + q);
                            const float2 ex = __fadd2_rn(X, nx0);
                            const float2 ey = __fadd2_rn(Y, nx1);
                            float2 d2 = __ffma2_rn(ey, ey, __fmul2_rn(ex, ex));
                            if (DIM == 3) {
                                const float2 ez = __fadd2_rn(*reinterpret_cast<const float2*>(tz + q), nx2);
                                d2 = __ffma2_rn(ez, ez, d2);
                            }
                            m |= (d2.x < reach2 ? 1u : 0u) << q;
                            m |= (d2.y < reach2 ? 1u : 0u) << (q + 1);
                        }
                    }
                    if constexpr (EXACT) {
                        if (n < 32) maybe &= (1u << n) - 1u;
                        while (maybe) {
                            const int q = __ffs(maybe) - 1;
                            maybe &= maybe - 1u;
                            if (exact_in_range<DIM>(t, d.xm[c0 + q])) m |= 1u << q;
                        }
                    }
                    if (n < 32) m &= (1u << n) - 1u;
                    const unsigned self = (unsigned)(t.i - c0);
                    if (self < 32u) m &= ~(1u << self);
                }
                if constexpr (Share::on) m = sh.take(sh.join(m));
                if constexpr (Split::on) {
                    // Append in order; a lane whose list is full (K entries)
                    // runs it there.  Its lists are then cut at every K-th
                    // neighbour of its own sequence, whatever the tiles and the
                    // warp's other targets, so its pair order (approaching,
                    // then receding, per cut) depends on its own candidates
                    // alone.  K is above the neighbour count of a lattice
                    // target (56 in 3-D, 20 in 2-D), so the cuts are rare and
                    // the lists run together after the walk.
                    auto append = [&](int q) {
                        const float4 p = tile[q], w = tilev[q];
                        float xv = (x0 - p.x) * (sp.vx - w.x) + (x1 - p.y) * (sp.vy - w.y);
                        if (DIM == 3) xv += (x2 - p.z) * (sp.vz - w.z);
                        if (xv < 0.0f) {
                            lst[cnt * 32 + lane] = (uint32_t)(c0 + q);
                            ++cnt;
                        } else {
                            ++nb;
                            lst[(K - nb) * 32 + lane] = (uint32_t)(c0 + q);
                        }
                    };
                    if (!__any_sync(SPH_FULL_MASK, cnt + nb > K - 32)) {
                        // the whole tile fits every list
                        while (m) {
                            append(__ffs(m) - 1);
                            m &= m - 1u;
                        }
                    } else {
                        while (true) {
                            while (m && cnt + nb < K) {
                                append(__ffs(m) - 1);
                                m &= m - 1u;
                            }
                            const bool full = cnt + nb == K;
                            if (!__any_sync(SPH_FULL_MASK, full)) break;
                            flush(full);
                        }
                    }
                    __syncwarp();
                } else {
                    while (m) {
                        lst[cnt * 32 + lane] = (uint32_t)(c0 + __ffs(m) - 1);
                        ++cnt;
                        m &= m - 1u;
                    }
                    __syncwarp();
                    // a list that could overflow on the next tile is run; a
                    // lane's pairs stay in walk order whatever the cut points
                    if (__any_sync(SPH_FULL_MASK, cnt > K - 32)) flush(true);
                }
            }
        }
    }
    flush(true);
}

// Distance helpers for the FP64 pair physics.
template <int DIM>
struct Geo {
    double dx[3], dr, rinv, r;
};
template <int DIM>
__device__ __forceinline__ Geo<DIM> geo(const double* xi, const double4& xj) {
    Geo<DIM> g;
    g.dx[0] = xi[0] - xj.x;
    g.dx[1] = xi[1] - xj.y;
    g.dx[2] = DIM == 3 ? xi[2] - xj.z : 0.0;
    g.dr = g.dx[0] * g.dx[0] + g.dx[1] * g.dx[1];
    if (DIM == 3) g.dr += g.dx[2] * g.dx[2];
    g.rinv = __double_as_longlong(g.dr) != 0 ? rsqrt(g.dr) : 0.0;   // dr is +0 or positive
    g.r = g.dr * g.rinv;
    return g;
}

// ---------------------------------------------------------------------------
// pass K: kernel gradient correction (kernelGradientCorrection.f90:8-51):
// A_i = sum_j (x_j - x_i)_e dW_d m_j / rho_j over neighbours whose
// (|Type| - 100) has the target's sign (every target is a solid), then the
// factors of the reference's pivoted elimination of A_i
// ---------------------------------------------------------------------------
template <int DIM>
struct PhysK {
    const Dev& d;
    double xi[3];
    KConst kc;
    int skf;
    double A[DIM][DIM];
    __device__ PhysK(const Dev& dd, const double4& x, double h, int i) : d(dd) {
        xi[0] = x.x; xi[1] = x.y; xi[2] = x.z;
        skf = d.skf;
        kc = kconst_of<DIM>(d, i, skf, h);
#pragma unroll
        for (int a = 0; a < DIM; ++a)
#pragma unroll
            for (int b = 0; b < DIM; ++b) A[a][b] = 0.0;
    }
    __device__ __forceinline__ void pair(int j) {
        if (abs(d.meta[j].x) < 100) return;
        const double4 xj = d.xm[j];
        Geo<DIM> g = geo<DIM>(xi, xj);
        const double gf = skf == 1 ? cubic_g_r(kc, g.r, g.rinv) : kernel_g(skf, kc, g.r * kc.hinv, g.rinv);
        const double Vj = d.eh[j].w;
#pragma unroll
        for (int a = 0; a < DIM; ++a)
#pragma unroll
            for (int e = 0; e < DIM; ++e) A[a][e] += ((-g.dx[e]) * (gf * g.dx[a])) * Vj;
    }
};

template <int DIM>
__global__ void __launch_bounds__(TPB, 4) pass_k_kernel(const Dev d) {
    constexpr int K = ListLen<DIM>::K;
    extern __shared__ uint32_t smem[];
    uint32_t* lst = smem + (threadIdx.x >> 5) * ListLen<DIM>::SLOT;
    const int i = blockIdx.x * TPB + threadIdx.x;
    const bool valid = i < d.n_real;
    const int ii = valid ? i : 0;
    const double4 xm = d.xm[ii];
    const double4 eh = d.eh[ii];
    const int4 meta = d.meta[ii];
    Target<DIM> t = make_target<DIM>(d, ii, xm, eh.y);
    PhysK<DIM> ph(d, xm, eh.y, ii);
    walk_lane<DIM, K>(d, t, valid && meta.w != -1, ph, lst, ExactAccept<DIM>{d, t});
    if (!valid) return;
    kgc_factor<DIM>(ph.A, d.kgc + (size_t)i * KGC_STRIDE);
}

// ---------------------------------------------------------------------------
// pass S: summation density (density.f90:10-80), before pass A so that every
// later pair term reads the summed densities
// ---------------------------------------------------------------------------
template <int DIM>
struct PhysS {
    const Dev& d;
    double xi[3];
    KConst kc;
    int skf;
    bool norm;
    double rho;  // sum_j m_j W_ij
    double wv;   // sum_j m_j / rho_j W_ij (normalisation)
    __device__ PhysS(const Dev& dd, const double4& x, double h, bool nrm, int i) : d(dd), norm(nrm) {
        xi[0] = x.x; xi[1] = x.y; xi[2] = x.z;
        skf = d.skf;
        kc = kconst_of<DIM>(d, i, skf, h);
        rho = 0.0;
        wv = 0.0;
    }
    __device__ __forceinline__ void pair(int j) {
        const double4 xj = d.xm[j];
        Geo<DIM> g = geo<DIM>(xi, xj);
        const double w = kernel_w(skf, kc, g.r * kc.hinv);
        rho = fma(xj.w, w, rho);
        if (norm) wv = fma(d.eh[j].w, w, wv);
    }
};

template <int DIM>
__global__ void __launch_bounds__(TPB, 4) pass_s_kernel(const Dev d) {
    constexpr int K = ListLen<DIM>::K;
    extern __shared__ uint32_t smem[];
    uint32_t* lst = smem + (threadIdx.x >> 5) * ListLen<DIM>::SLOT;
    float4* tile = reinterpret_cast<float4*>(lst + K * 32);
    const int i = blockIdx.x * TPB + threadIdx.x;
    const bool valid = i < d.n_real;
    const int ii = valid ? i : 0;
    const double4 xm = d.xm[ii];
    const double4 eh = d.eh[ii];
    const int4 meta = d.meta[ii];
    // Shepard normalisation where divergencePosition (last step) < 1.5
    const bool norm = (d.flags & SPH_F_NORM_DENSITY) && d.dxp[ii] < 1.5;
    Target<DIM> t = make_target<DIM>(d, ii, xm, eh.y);
    PhysS<DIM> ph(d, xm, eh.y, norm, ii);
    walk_lane<DIM, K>(d, t, valid && meta.w != -1, ph, lst, ExactAccept<DIM>{d, t});
    if (!valid) return;
    const double self = kernel_w(ph.skf, ph.kc, 0.0);
    double rho = xm.w * self + ph.rho;
    if (norm) rho = rho / (eh.w * self + ph.wv);
    d.rsum[i] = rho;
}

// The summed densities replace rho (and m / rho, and their FP32 mirrors).
__global__ void density_apply_kernel(const Dev d) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.n_real) return;
    const double rho = d.rsum[s];
    double4 vr = d.vr[s];
    vr.w = rho;
    d.vr[s] = vr;
    double4 eh = d.eh[s];
    eh.w = d.xm[s].w / rho;
    d.eh[s] = eh;
    if (d.precision == SPH_PREC_MIXED) {
        float4 v = d.vf4[s];
        v.w = (float)rho;
        d.vf4[s] = v;
        float4 e = d.ef4[s];
        e.z = (float)eh.w;
        d.ef4[s] = e;
    } else if (d.precision == SPH_PREC_DF64) {
        const DF r = df_from(rho), V = df_from(eh.w);
        d.vd0[s].w = r.hi;
        d.vd1[s].w = r.lo;
        float4 e = d.ed0[s];
        e.x = V.hi;
        e.y = V.lo;
        d.ed0[s] = e;
    }
}

// ---------------------------------------------------------------------------
// pass A: density rate / divergence / velocity gradient
// ---------------------------------------------------------------------------
template <int DIM, bool KGC = false, bool XS = false>
struct PhysA {
    const Dev& d;
    double xi[3], vi[3];
    KConst kc;
    int skf;
    const double* kf = nullptr;  // the target's kernel-correction factors
    double G[DIM][DIM];  // sum_j V_j (v_j - v_i)_a dW/dx_b
    double sdx;          // sum_j V_j dx . dW
    int nn;
    static constexpr bool xsph = XS;   // aver_velo (correctVelocity.f90:7-44)
    double rhoi;
    double axs[DIM];     // sum_j 2 eps m_j (v_i - v_j) W_ij / (rho_i + rho_j)
    __device__ PhysA(const Dev& dd, const double4& x, const double4& v, double h, int i) : d(dd) {
        xi[0] = x.x; xi[1] = x.y; xi[2] = x.z;
        vi[0] = v.x; vi[1] = v.y; vi[2] = v.z;
        rhoi = v.w;
#pragma unroll
        for (int a = 0; a < DIM; ++a) axs[a] = 0.0;
        skf = d.skf;
        kc = kconst_of<DIM>(d, i, skf, h);
#pragma unroll
        for (int a = 0; a < DIM; ++a)
#pragma unroll
            for (int b = 0; b < DIM; ++b) G[a][b] = 0.0;
        sdx = 0.0;
        nn = 0;
    }
    __device__ __forceinline__ void pair(int j) {
        const double4 xj = d.xm[j];
        const double4 vj = d.vr[j];
        const double Vj = d.eh[j].w;
        Geo<DIM> g = geo<DIM>(xi, xj);
        const double gf = skf == 1 ? cubic_g_r(kc, g.r, g.rinv) : kernel_g(skf, kc, g.r * kc.hinv, g.rinv);
        if constexpr (KGC) {
            // corrected gradient: not parallel to dx any more
            double gr[DIM];
#pragma unroll
            for (int a = 0; a < DIM; ++a) gr[a] = gf * g.dx[a];
            kgc_apply<DIM>(kf, gr);
            double u[DIM], xg = 0.0;
#pragma unroll
            for (int a = 0; a < DIM; ++a) {
                u[a] = Vj * (cmp(vj, a) - vi[a]);
                xg = fma(g.dx[a], gr[a], xg);
            }
#pragma unroll
            for (int a = 0; a < DIM; ++a)
#pragma unroll
                for (int b = 0; b < DIM; ++b) G[a][b] = fma(u[a], gr[b], G[a][b]);
            sdx = fma(Vj, xg, sdx);
        } else {
            // V_j (v_j - v_i)_a dW_b = (V_j g (v_j - v_i)_a) dx_b
            const double vg = Vj * gf;
            double u[DIM];
#pragma unroll
            for (int a = 0; a < DIM; ++a) u[a] = vg * (cmp(vj, a) - vi[a]);
#pragma unroll
            for (int a = 0; a < DIM; ++a)
#pragma unroll
                for (int b = 0; b < DIM; ++b) G[a][b] = fma(u[a], g.dx[b], G[a][b]);
            sdx = fma(vg, g.dr, sdx);
        }
        ++nn;
        if constexpr (XS) {
            const double W = kernel_w(skf, kc, g.r * kc.hinv);
            const double f = (((d.xsph_eps * 2) * xj.w) / (rhoi + vj.w)) * W;
#pragma unroll
            for (int a = 0; a < DIM; ++a) axs[a] = fma(f, vi[a] - cmp(vj, a), axs[a]);
        }
    }
    // the sums of the L lanes of a target's group (LaneShare)
    __device__ __forceinline__ void lane_sums(int L) {
#pragma unroll
        for (int a = 0; a < DIM; ++a)
#pragma unroll
            for (int b = 0; b < DIM; ++b) G[a][b] = lane_sum(G[a][b], L);
        sdx = lane_sum(sdx, L);
        nn = lane_sum(nn, L);
        if constexpr (XS) {
#pragma unroll
            for (int a = 0; a < DIM; ++a) axs[a] = lane_sum(axs[a], L);
        }
    }
};

// Double-float geometry of a pair (DF64 mode): dx = x_i - x_j from the
// positions relative to the grid origin, r^2, 1/r, r and the cubic-spline
// gradient factor (the forms of cubic_g_r).
template <int DIM>
struct GeoD {
    DF dx[3], dr, rinv, r, gf;
};
struct KConstD {
    DF A1, B1, C1, C2, C3, h;
};
__device__ __forceinline__ KConstD make_kconst_d(const KConst& k) {
    return KConstD{df_from(k.A1), df_from(k.B1), df_from(k.C1), df_from(k.C2), df_from(k.C3), df_from(k.h)};
}
template <int DIM>
__device__ __forceinline__ GeoD<DIM> geo_d(const DF* xi, const float4& a0, const float4& a1, const KConstD& k) {
    GeoD<DIM> g;
    g.dx[0] = df_sub(xi[0], DF{a0.x, a1.x});
    g.dx[1] = df_sub(xi[1], DF{a0.y, a1.y});
    g.dx[2] = DIM == 3 ? df_sub(xi[2], DF{a0.z, a1.z}) : DF{0.0f, 0.0f};
    g.dr = df_mul(g.dx[0], g.dx[0]);
    g.dr = df_fma(g.dx[1], g.dx[1], g.dr);
    if (DIM == 3) g.dr = df_fma(g.dx[2], g.dx[2], g.dr);
    g.rinv = g.dr.hi > 0.0f ? df_rsqrt(g.dr) : DF{0.0f, 0.0f};
    g.r = df_mul(g.dr, g.rinv);
    const bool inner = g.r.hi < k.h.hi || (g.r.hi == k.h.hi && g.r.lo < k.h.lo);
    g.gf = inner ? df_fma(k.B1, g.r, k.A1) : df_fma(k.C1, g.rinv, df_fma(k.C2, g.r, k.C3));
    return g;
}

// pass A pair physics in double-float (fluid targets, cubic spline): the
// sums of PhysA; after the walk finalize() leaves them as doubles in the
// members the FP64 epilogue reads.  XS adds the XSPH sum (correctVelocity.f90:
// 7-44) with the cubic kernel value W(q) (kernel.f90:30-71) in double-float.
template <int DIM, bool XS>
struct PhysAd {
    const Dev& d;
    DF xi[3], vi[3];
    KConstD kc;
    DFAcc Gd[DIM][DIM], sdxd;
    double G[DIM][DIM];
    double sdx;
    int nn = 0;
    static constexpr bool xsph = XS;
    double axs[DIM];
    // XS only: rho_i, 1/h, the kernel factor and factor/6, 2/3, 2 eps_XSPH
    DF rhoi, hinv, wf, wf6, two3, eps2;
    DFAcc axd[DIM];
    __device__ PhysAd(const Dev& dd, const double4&, const double4&, double h, int i) : d(dd) {
        const KConst k = kconst_of<DIM>(d, i, 1, h);
        kc = make_kconst_d(k);
        if constexpr (XS) {
            hinv = df_from(k.hinv);
            wf = df_from(k.factor);
            wf6 = df_from(k.factor * (1.0 / 6.0));
            two3 = df_from(2.0 / 3.0);
            eps2 = df_from(d.xsph_eps * 2);
        }
#pragma unroll
        for (int a = 0; a < DIM; ++a) axs[a] = 0.0;
    }
    __device__ __forceinline__ void target(int i) {
        const float4 a0 = d.pd0[i], a1 = d.pd1[i], v0 = d.vd0[i], v1 = d.vd1[i];
        xi[0] = DF{a0.x, a1.x}; xi[1] = DF{a0.y, a1.y}; xi[2] = DF{a0.z, a1.z};
        vi[0] = DF{v0.x, v1.x}; vi[1] = DF{v0.y, v1.y}; vi[2] = DF{v0.z, v1.z};
        if constexpr (XS) rhoi = DF{v0.w, v1.w};
    }
    __device__ __forceinline__ void pair(int j) {
        const float4 a0 = d.pd0[j], a1 = d.pd1[j], v0 = d.vd0[j], v1 = d.vd1[j];
        const float4 e0 = d.ed0[j];
        const GeoD<DIM> g = geo_d<DIM>(xi, a0, a1, kc);
        const DF vg = df_mul(DF{e0.x, e0.y}, g.gf);
        const DF vj[3] = {DF{v0.x, v1.x}, DF{v0.y, v1.y}, DF{v0.z, v1.z}};
        DF u[DIM];
#pragma unroll
        for (int a = 0; a < DIM; ++a) u[a] = df_mul(vg, df_sub(vj[a], vi[a]));
#pragma unroll
        for (int a = 0; a < DIM; ++a)
#pragma unroll
            for (int b = 0; b < DIM; ++b) Gd[a][b].add_prod(u[a], g.dx[b]);
        sdxd.add_prod(vg, g.dr);
        ++nn;
        if constexpr (XS) {
            // W(q): q < 1: factor ((2/3 - q^2) + q^3 / 2); 1 <= q <= 2:
            // factor / 6 (2 - q)^3 (a neighbour has q < 2)
            const DF q = df_mul(g.r, hinv);
            const DF q2 = df_mul(q, q);
            const DF w1 = df_mul(wf, df_add(df_sub(two3, q2), df_mul_f(df_mul(q2, q), 0.5f)));
            const DF t = df_add_f(df_neg(q), 2.0f);
            const DF w2 = df_mul(wf6, df_mul(df_mul(t, t), t));
            const bool inner = q.hi < 1.0f || (q.hi == 1.0f && q.lo < 0.0f);
            const DF W = inner ? w1 : w2;
            // ((2 eps) m_j / (rho_i + rho_j)) W (v_i - v_j)
            const DF f = df_mul(df_mul(df_mul(eps2, DF{a0.w, a1.w}), df_rcp(df_add(rhoi, DF{v0.w, v1.w}))), W);
#pragma unroll
            for (int a = 0; a < DIM; ++a) axd[a].add_prod(f, df_sub(vi[a], vj[a]));
        }
    }
    __device__ __forceinline__ void finalize() {
#pragma unroll
        for (int a = 0; a < DIM; ++a)
#pragma unroll
            for (int b = 0; b < DIM; ++b) G[a][b] = Gd[a][b].to_double();
        sdx = sdxd.to_double();
        if constexpr (XS) {
#pragma unroll
            for (int a = 0; a < DIM; ++a) axs[a] = axd[a].to_double();
        }
    }
};

// LS: 2^lane_shift lanes per target (LaneShare); the first lane of each
// group writes the results.
template <int DIM, bool SOLID, bool KGC = false, bool DFM = false, bool XS = false, bool LS = false>
__global__ void __launch_bounds__(TPB, 4) pass_a_kernel(const Dev d, int want_strain) {
    static_assert(!LS || (!KGC && !DFM), "lanes per target: the plain FP64 form");
    constexpr int K = ListLen<DIM, true>::K;
    constexpr int D2 = DIM * DIM;
    extern __shared__ uint32_t smem[];
    uint32_t* lst = smem + (threadIdx.x >> 5) * ListLen<DIM, true>::SLOT;
    float4* tile = reinterpret_cast<float4*>(lst + K * 32);
    const int gt = blockIdx.x * TPB + threadIdx.x;
    const int lsh = LS ? d.lane_shift : 0;
    const int i = gt >> lsh;
    const bool valid = i < d.n_real;
    const int ii = valid ? i : 0;
    const double4 xm = d.xm[ii];
    const double4 vr = d.vr[ii];
    const double4 eh = d.eh[ii];
    const int4 meta = d.meta[ii];
    Target<DIM> t = make_target<DIM>(d, ii, xm, eh.y);
    using PA = std::conditional_t<DFM, PhysAd<DIM, XS>, PhysA<DIM, KGC, XS>>;
    PA ph(d, xm, vr, eh.y, ii);
    if constexpr (KGC) ph.kf = d.kgc + (size_t)ii * KGC_STRIDE;
    if constexpr (DFM) ph.target(ii);
    if constexpr (LS) {
        const LaneShare share{gt & ((1 << lsh) - 1), (1 << lsh) - 1};
        walk_tiled<DIM, K, PA, true, NoSplit, LaneShare>(d, t, valid && meta.w != -1, ph, lst, tile, 0.0f,
                                                         NoSplit{}, share);
        ph.lane_sums(1 << lsh);
        if (share.sub != 0) return;
    } else {
        walk_tiled<DIM, K, PA, true>(d, t, valid && meta.w != -1, ph, lst, tile, 0.0f);
    }
    if constexpr (DFM) ph.finalize();
    if (!valid) return;

    const double rho = vr.w;
    const int type = meta.x;
    const bool visc = d.flags & SPH_F_VISCOSITY;
    const DevMaterial* m = material_of(d, inst_of(d, i), type);
    const double eta = (visc && m) ? m->eta : 0.0;
    double divv = 0.0;
#pragma unroll
    for (int a = 0; a < DIM; ++a) divv += ph.G[a][a];
    const double divx = -ph.sdx;
    double p = d.pa4[i].y, c = eh.z;
    double edot[DIM][DIM];
    double tds = 0.0;
    const double rho2 = rho * rho;
    // one division for the epilogue's 1 / rho, 1 / rho^2 (each within an ulp
    // or two of the divisions it replaces; a division costs about ten FP64
    // FMAs on this GPU)
    const double irho = 1.0 / rho;
    const double irho2 = irho * irho;
    const bool solid = SOLID && is_solid_type(type);
    if (!solid) {
        // fluid strain rate, internalForce.f90:56-77 (quirk: off-diagonals are
        // 2 sum V dv_a dW_b, not symmetrised)
#pragma unroll
        for (int a = 0; a < DIM; ++a)
#pragma unroll
            for (int b = 0; b < DIM; ++b)
                edot[a][b] = visc ? 2.0 * ph.G[a][b] - (a == b ? (2.0 / 3.0) * divv : 0.0) : 0.0;
        if (visc) {
            double s = 0.0;
#pragma unroll
            for (int b = 0; b < DIM; ++b)
#pragma unroll
                for (int a = 0; a < DIM; ++a) s += edot[a][b] * edot[a][b];
            tds = ((0.5 * eta) * irho) * s;
        }
        fluid_eos(m, rho, eh.x, p, c);
        if (SOLID) {
#pragma unroll
            for (int k = 0; k < D2; ++k) d.sig[(size_t)i * D2 + k] = 0.0;
            if (DIM == 2) d.ras[i] = make_double4(0, 0, 0, 0);
        }
    } else {
        // solid strain / rotation rate (internalForce.f90:82-95), deviatoric
        // stress rate (Jaumann) and stress (:137-180)
        double rot[DIM][DIM];
#pragma unroll
        for (int a = 0; a < DIM; ++a)
#pragma unroll
            for (int b = 0; b < DIM; ++b) {
                edot[a][b] = visc ? 0.5 * (ph.G[a][b] + ph.G[b][a]) : 0.0;
                rot[a][b] = visc ? 0.5 * (ph.G[a][b] - ph.G[b][a]) : 0.0;
            }
        double tr = 0.0;
#pragma unroll
        for (int a = 0; a < DIM; ++a) tr += edot[a][a];
        tr = tr / 3;  // trace/3 even in 2-D (quirk Q2)
        double eb[DIM][DIM], S[DIM][DIM];
        const double* sh = d.shear + (size_t)i * D2;
#pragma unroll
        for (int b = 0; b < DIM; ++b)
#pragma unroll
            for (int a = 0; a < DIM; ++a) {
                S[a][b] = sh[b * DIM + a];
                eb[a][b] = edot[a][b] - (a == b ? tr : 0.0);
            }
        double s = 0.0;
#pragma unroll
        for (int b = 0; b < DIM; ++b)
#pragma unroll
            for (int a = 0; a < DIM; ++a) s += S[a][b] * eb[a][b];
        tds = s * irho;
        solid_eos(m, rho, eh.x, p);
        const double G2 = 2.0 * eta;
        double* ds = d.dsdt + (size_t)i * D2;
        double* sg = d.sig + (size_t)i * D2;
#pragma unroll
        for (int a = 0; a < DIM; ++a)
#pragma unroll
            for (int b = 0; b < DIM; ++b) {
                double v = G2 * eb[a][b];
#pragma unroll
                for (int k = 0; k < DIM; ++k) v += S[a][k] * rot[b][k] + S[b][k] * rot[a][k];
                ds[b * DIM + a] = v;
                double st = S[a][b] - (a == b ? p : 0.0);
                sg[b * DIM + a] = st * irho2;
            }
        if (DIM == 2) {
            // artificial stress tensor R_i (artificialTerm.f90:42-69)
            double4 R = make_double4(0, 0, 0, 0);
            if (type >= 100) {
                constexpr double PI = 3.141592653589793238462643383279502884;
                const double s11 = S[0][0] - p, s22 = S[1][1] - p, s12 = S[0][1], s21 = S[1][0];
                const double aux = s11 - s22;
                const double th = aux == 0.0 ? 0.5 * PI : 0.5 * atan((s12 + s21) / aux);
                double sn, cs;
                sincos(th, &sn, &cs);
                const double ps0 = (cs * cs) * s11 + (sn * sn) * s22 + 2 * sn * cs * s12;
                const double ps1 = (sn * sn) * s11 + (cs * cs) * s22 - 2 * sn * cs * s12;
                const double T0 = ps0 > 0 ? -(d.as_eps * ps0 / rho2) : 0.0;
                const double T1 = ps1 > 0 ? -(d.as_eps * ps1 / rho2) : 0.0;
                R.x = (cs * cs) * T0 + (sn * sn) * T1;
                R.y = (sn * sn) * T0 + (cs * cs) * T1;
                R.z = sn * cs * (T0 - T1);
            }
            d.ras[i] = R;
        }
    }
    // (eta edot - p I) / rho^2 of this particle, read by its fluid neighbours
    // in pass B (a solid's viscous part is dropped under
    // SPH_F_FSI_FLUID_VISCOUS); under SPH = 1 / 3 eta edot alone
    double* tt = d.tt + (size_t)i * D2;
    const bool sph2 = d.pa_sph == 2;
    const bool drop_tt = sph2 && solid && (d.flags & SPH_F_FSI_FLUID_VISCOUS);
    const double pr2 = p * irho2;
#pragma unroll
    for (int b = 0; b < DIM; ++b)
#pragma unroll
        for (int a = 0; a < DIM; ++a) {
            const double v = drop_tt ? 0.0 : (sph2 ? (eta * edot[a][b]) * irho2 : eta * edot[a][b]);
            tt[b * DIM + a] = (sph2 && a == b) ? v - pr2 : v;
        }
    if constexpr (DFM) {
#pragma unroll
        for (int k = 0; k < D2; ++k) {
            const DF v = df_from(tt[k]);
            d.ttd[(size_t)i * D2 + k] = make_float2(v.hi, v.lo);
        }
        const DF P = df_from(pr2), cc = df_from(c);
        d.ed1[i] = make_float4(cc.hi, cc.lo, P.hi, P.lo);
    }
    if (want_strain) {
        double* st = d.strain + (size_t)i * D2;
#pragma unroll
        for (int b = 0; b < DIM; ++b)
#pragma unroll
            for (int a = 0; a < DIM; ++a) st[b * DIM + a] = edot[a][b];
    }
    d.pa4[i] = make_double4(pr2, p, divv, divx);
    d.tds[i] = tds;
    if (c != eh.z) d.eh[i].z = c;
    if (d.dxp) d.dxp[i] = divx;
    if (d.pa_sph == 3) {
        // con_density_riemann wrote the rate (pass R)
    } else if (!(d.flags & SPH_F_SUM_DENSITY)) {
        d.dvr[i].w = -rho * divv;  // con_density
    } else {
        d.dvr[i].w = 0.0;
    }
    if constexpr (XS) {  // no correction where Boundary == 1
        double v[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int a = 0; a < DIM; ++a) v[a] = meta.y == 1 ? 0.0 : -ph.axs[a];
        d.aver[i] = make_double4(v[0], v[1], v[2], 0.0);
    }
    d.nneigh[i] = ph.nn;
}

// ---------------------------------------------------------------------------
// pass B: forces
// ---------------------------------------------------------------------------
// Squared distance beyond which no external pair term can be non-zero (with
// a relative margin far above rounding): wall repulsion needs r < r0, the
// contact force r < delta, the multiphase penalty r <= (h_i + h_j) / 2.
__device__ __forceinline__ float ext_reach2(const Inst& I, bool wall, float hi, float hj) {
    if (wall) return I.ext_wall_r2;
    const float r = fmaxf(I.ext_delta, 0.5f * (hi + hj)) * 1.0001f;
    return r * r;
}

// The parameters of the external pair terms, gathered where a pair needs them.
struct ExtPrm {
    double wall_r0, contact_delta, wall_fs, wall_p1, wall_p2, pen_factor, pen_n1, pen_n2;
};
__device__ __forceinline__ ExtPrm ext_prm(const Dev& d, const Inst& I) {
    return ExtPrm{I.wall_r0, I.contact_delta, d.wall_fs, d.wall_p1, d.wall_p2, d.pen_factor, d.pen_n1, d.pen_n2};
}

// externalForce.f90:103-173 for one pair (i real, j any, h_j the
// neighbour's smoothing length); r is recomputed exactly as the reference
// computes it.  Adds to aex.
template <int DIM>
__device__ __forceinline__ void external_terms(const ExtPrm& e, const double* xi, double hi, double ci, int typei,
                                               int tj, double hj, const double4& xj, double* aex) {
    const bool wallpair = typei > 0 && tj < 0;
    const bool phase = typei != tj && typei > 0 && tj > 0;
    if (!wallpair && !phase) return;
    double dx[3];
    dx[0] = __dsub_rn(xi[0], xj.x);
    double dr = __dmul_rn(dx[0], dx[0]);
    dx[1] = __dsub_rn(xi[1], xj.y);
    dr = __dadd_rn(dr, __dmul_rn(dx[1], dx[1]));
    if (DIM == 3) { dx[2] = __dsub_rn(xi[2], xj.z); dr = __dadd_rn(dr, __dmul_rn(dx[2], dx[2])); }
    const double r = __dsqrt_rn(dr);
    const double r2 = r * r;
    // each term adds f dx / r^2: one division per term, then products
    if (wallpair && r < e.wall_r0) {
        const double t = e.wall_r0 / r;
        const double f = e.wall_fs * (pow_int_or_real(t, e.wall_p1) - pow_int_or_real(t, e.wall_p2));
        const double fr = f / r2;
#pragma unroll
        for (int a = 0; a < DIM; ++a) aex[a] += fr * dx[a];
    }
    if (phase) {
        if (typei < 100 && tj < 100) {  // multiphase penalty
            const double pe = (hi + hj) / (2 * r);
            if (pe >= 1) {
                const double f = e.pen_factor * (pow(pe, e.pen_n1) - pow(pe, e.pen_n2));
                const double fr = f / r2;
#pragma unroll
                for (int a = 0; a < DIM; ++a) aex[a] += fr * dx[a];
            }
        } else if (!(typei > 100 && tj > 100)) {  // fluid-solid contact
            const double eta = r / 0.75 / ((hi + hj) * 0.5);
            double chi = 1 - r / e.contact_delta;
            if (chi < 0 || chi > 1) chi = 0;
            double fc;
            if (eta <= 0 || eta >= 2) fc = 0;
            else if (eta <= 2.0 / 3) fc = 2.0 / 3;
            else if (eta <= 1) fc = 2 * eta - 1.5 * eta * eta;
            else fc = 0.5 * ((2 - eta) * (2 - eta));
            const double f = (double)0.01f * (ci * ci) * chi * fc;
            const double fr = f / r2;
#pragma unroll
            for (int a = 0; a < DIM; ++a) aex[a] += fr * dx[a];
        }
    }
}

// external_terms out of line, for the FP64 pair loops: they call it for the
// few pairs within reach, and the loop body keeps none of its registers.
// Takes the target's a_ext and returns it with the pair's term added.
template <int DIM>
__device__ __noinline__ double3 external_terms_call(const ExtPrm e, double xi0, double xi1, double xi2, double hi,
                                                    double ci, int typei, int tj, double hj, double4 xj, double3 acc) {
    const double xi[3] = {xi0, xi1, xi2};
    double aex[3] = {acc.x, acc.y, acc.z};
    external_terms<DIM>(e, xi, hi, ci, typei, tj, hj, xj, aex);
    return make_double3(aex[0], aex[1], aex[2]);
}
// The call site of the FP64 pair loops: gathers the parameters and h_j, and
// adds the pair's term to aex through the out-of-line call.
template <int DIM>
__device__ __forceinline__ void external_pair(const Dev& d, const Inst& I, const double* xi, double hi, double ci,
                                              int typei, int j, int tj, const double4& xj, double* aex) {
    const double3 r = external_terms_call<DIM>(ext_prm(d, I), xi[0], xi[1], DIM > 2 ? xi[2] : 0.0, hi, ci, typei,
                                               tj, d.eh[j].y, xj, make_double3(aex[0], aex[1], DIM > 2 ? aex[2] : 0.0));
    aex[0] = r.x;
    aex[1] = r.y;
    if (DIM > 2) aex[2] = r.z;
}

// SCH: the momentum / energy form of the fluid targets (internalForce.f90:194):
// 2, P/rho^2 form (the default); 1, (P_i + P_j) / (rho_i rho_j); 3, the PVRS
// Riemann solver.  Under 1 and 3 solid targets get no internal force, and
// the sums use V_j = m_j / rho_j with a final 1 / rho_i; the tensors in tt
// are eta edot without the 1 / rho^2.
template <int DIM, bool SOLID, bool KGC = false, int SCH = 2, bool AH = false>
struct PhysB {
    static_assert(SCH == 2 || !KGC, "kernel correction is paired with SPH = 2 only");
    static_assert(!AH || (SCH == 2 && !KGC), "artificial heat is paired with SPH = 2 without correction");
    const Dev& d;
    uint32_t terms;
    // AH: artificial heat (artificialHeat.f90:6-56): the target's
    // q = 0.1 h c + h^2 (|div v| - div v) and e, and the sum of the pair terms
    double qi = 0.0, ei = 0.0, ah = 0.0;
    double xi[3], vi[3];
    double hi, rhoi, ci, Pi;
    int typei;
    bool solid_i;
    KConst kc;
    int skf;
    double wd;       // W(delta_p, h_i) of the artificial stress
    double4 Ri;
    const Inst* I;   // the target's system
    const double* kf = nullptr;  // the target's kernel-correction factors
    // accumulators
    double ap[DIM], sw[DIM], ein, aav[DIM], eav, aex[DIM], aas[DIM];

    __device__ PhysB(const Dev& dd, uint32_t tm, const double4& x, const double4& v, const double4& e,
                     double P, int type, const Inst* inst, int i) : d(dd), terms(tm), I(inst) {
        xi[0] = x.x; xi[1] = x.y; xi[2] = x.z;
        vi[0] = v.x; vi[1] = v.y; vi[2] = v.z;
        hi = e.y; rhoi = v.w; ci = e.z; Pi = P; typei = type;
        solid_i = SOLID && is_solid_type(type);
        skf = d.skf;
        kc = kconst_of<DIM>(d, i, skf, hi);
        wd = 1.0;
        Ri = make_double4(0, 0, 0, 0);
#pragma unroll
        for (int a = 0; a < DIM; ++a) { ap[a] = 0; sw[a] = 0; aav[a] = 0; aex[a] = 0; aas[a] = 0; }
        ein = 0; eav = 0;
        // gravity is set before the pair terms are added (externalForce.f90:27-59)
        if ((terms & SPH_TERM_EXTERNAL) && (d.flags & SPH_F_GRAVITY) &&
            !((d.flags & SPH_F_GRAVITY_SKIP_SOLIDS) && type > 100))
            aex[DIM - 1] = d.gravity;
    }

    // AV constants (artificialViscosity.f90:75-78), the solid row for
    // Type > 100.  They are read from the kernel parameters where they are
    // used, so a fluid kernel holds none of them in registers over the walk.
    __device__ __forceinline__ bool av_solid() const { return SOLID && typei > 100; }
    __device__ __forceinline__ double alpha() const { return av_solid() ? d.av_alpha_solid : d.av_alpha; }
    __device__ __forceinline__ double beta() const { return av_solid() ? d.av_beta_solid : d.av_beta; }
    __device__ __forceinline__ double alpha_h() const { return av_solid() ? d.av_alpha_h_solid : d.av_alpha_h; }

    __device__ __forceinline__ void pair(int j) {
        const double4 xj = d.xm[j];
        const double4 vj = d.vr[j];
        Geo<DIM> g = geo<DIM>(xi, xj);
        // the cubic spline reads kc; the other kernels, and the artificial
        // stress, rebuild their constants from h_i where they are used, so
        // that the walk keeps only the cubic's in registers
        const double gf = skf == 1 ? cubic_g_r(kc, g.r, g.rinv) : kernel_g_of(g);
        const double mj = xj.w;
        double w[DIM], dv[DIM], gr[DIM];
        double dvw = 0.0, xv = 0.0;
#pragma unroll
        for (int a = 0; a < DIM; ++a) {
            dv[a] = vi[a] - cmp(vj, a);
            xv = fma(g.dx[a], dv[a], xv);
        }
        if constexpr (KGC) {
#pragma unroll
            for (int a = 0; a < DIM; ++a) gr[a] = gf * g.dx[a];
            kgc_apply<DIM>(kf, gr);
#pragma unroll
            for (int a = 0; a < DIM; ++a) {
                w[a] = mj * gr[a];
                dvw = fma(dv[a], w[a], dvw);
            }
        } else {
            // m_j dW = (m_j g) dx, so dv . m_j dW = (m_j g) (dx . dv)
            const double mg = mj * gf;
#pragma unroll
            for (int a = 0; a < DIM; ++a) w[a] = mg * g.dx[a];
            dvw = mg * xv;
        }
        if constexpr (SCH != 2) {
            if ((terms & SPH_TERM_INTERNAL) && !solid_i) internal_sch(j, g, gf, vj);
        } else if (terms & SPH_TERM_INTERNAL) {
            const double Pj = d.pa4[j].x;
            if (!solid_i) {
                // sum_j (T_j - P_j I) m_j dW, the pressure folded into the
                // diagonal of tt; the target's (T_i - P_i I) sum_j m_j dW is
                // applied once after the walk
                const double* Tj = d.tt + (size_t)j * DIM * DIM;
#pragma unroll
                for (int a = 0; a < DIM; ++a) {
                    double t = ap[a];
#pragma unroll
                    for (int b = 0; b < DIM; ++b) t = fma(Tj[b * DIM + a], w[b], t);
                    ap[a] = t;
                }
            } else {
                const double* Sj = d.sig + (size_t)j * DIM * DIM;
#pragma unroll
                for (int a = 0; a < DIM; ++a) {
                    double t = 0.0;
#pragma unroll
                    for (int b = 0; b < DIM; ++b) t = fma(Sj[b * DIM + a], w[b], t);
                    ap[a] += t;
                }
            }
#pragma unroll
            for (int a = 0; a < DIM; ++a) sw[a] += w[a];
            ein = fma(Pi + Pj, dvw, ein);
        }
        // approaching pairs; signbit also takes xv = -0, whose PI is a zero
        if ((terms & SPH_TERM_ARTI_VISC) && signbit(xv)) {
            const double4 ej = d.eh[j];
            double PI;
            const double beta = this->beta();
            if (beta == 0.0) {
                // PI = -alpha c phi / rho = -(alpha/2) (c_i+c_j)(h_i+h_j) x.v / (D (rho_i+rho_j))
                // with D = r^2 + (psi/2)^2 (h_i+h_j)^2
                const double sh = hi + ej.y;
                const double D = fma(d.av_psi_q * sh, sh, g.dr);
                PI = (alpha_h() * (ci + ej.z)) * (sh * xv) * rcp_nr(D * (rhoi + vj.w));
            } else {
                const double hij = 0.5 * (hi + ej.y);
                const double rij = 0.5 * (rhoi + vj.w);
                const double cij = 0.5 * (ci + ej.z);
                // PI = (beta phi - alpha c) phi / rho, phi = h x.v / D, with one
                // division: PI = hx (beta hx - alpha c D) / (D^2 rho)
                const double ph = d.av_psi * hij;
                const double D = fma(ph, ph, g.dr);
                const double hx = hij * xv;
                PI = hx * fma(beta, hx, -(alpha() * cij) * D) * rcp_nr((D * D) * rij);
            }
#pragma unroll
            for (int a = 0; a < DIM; ++a) aav[a] = fma(-PI, w[a], aav[a]);
            eav = fma(PI, dvw, eav);   // the 1/2 is applied after the walk
        }
        if constexpr (AH) {
            if (terms & SPH_TERM_ARTI_HEAT) {
                // q_ij (x_ij . dW) / (rho_ij (r^2 + 0.01 h_ij^2)), averages of the
                // pair; x_ij . dW = g r^2; the neighbour's div v is this step's
                // (0 for walls)
                const double4 ej = d.eh[j];
                const double divj = d.pa4[j].z;
                const double qj = (0.1 * ej.y) * ej.z + (ej.y * ej.y) * (fabs(divj) - divj);
                const double qij = 0.5 * (qi + qj);
                const double hij = 0.5 * (hi + ej.y);
                const double rij = 0.5 * (rhoi + vj.w);
                const double aux = qij * (gf * g.dr) / (rij * (g.dr + 0.01 * (hij * hij)));
                ah = fma((2.0 * mj) * aux, ei - ej.x, ah);
            }
        }
        if (terms & (SPH_TERM_EXTERNAL | SPH_TERM_ARTI_STRESS)) {
            const int tj = d.meta[j].x;
            if ((terms & SPH_TERM_EXTERNAL) && typei > 0 && (tj < 0 || tj != typei) &&
                le_pos(g.dr, f2d(ext_reach2(*I, tj < 0, d2f(hi), d2f(d.eh[j].y)))))
                external(j, tj, xj);
            if (SOLID && DIM == 2 && (terms & SPH_TERM_ARTI_STRESS) && tj >= 100) {
                const KConst kx = make_kconst<DIM>(skf, hi);
                const double W = kernel_w(skf, kx, g.r * kx.hinv);
                const double F = pow_int_or_real(W / wd, d.as_n);
                const double4 Rj = d.ras[j];
                const double r00 = Ri.x + Rj.x, r11 = Ri.y + Rj.y, r01 = Ri.z + Rj.z;
                const double gx = KGC ? gr[0] : gf * g.dx[0], gy = KGC ? gr[1] : gf * g.dx[1];
                aas[0] += (mj * F) * (r00 * gx + r01 * gy);
                aas[DIM > 1 ? 1 : 0] += (mj * F) * (r01 * gx + r11 * gy);
            }
        }
    }

    __device__ __forceinline__ void external(int j, int tj, const double4& xj) {
        external_pair<DIM>(d, *I, xi, hi, ci, typei, j, tj, xj, aex);
    }

    // LaneShare: the other lanes of a group start their external sum at 0
    // (the group's first lane holds the gravity), and after the walk every
    // lane takes the group's sums
    __device__ __forceinline__ void lane_start(int sub) {
        if (sub != 0) {
#pragma unroll
            for (int a = 0; a < DIM; ++a) aex[a] = 0.0;
        }
    }
    __device__ __forceinline__ void lane_sums(int L) {
#pragma unroll
        for (int a = 0; a < DIM; ++a) {
            ap[a] = lane_sum(ap[a], L);
            sw[a] = lane_sum(sw[a], L);
            aav[a] = lane_sum(aav[a], L);
            aex[a] = lane_sum(aex[a], L);
            aas[a] = lane_sum(aas[a], L);
        }
        ein = lane_sum(ein, L);
        eav = lane_sum(eav, L);
        if constexpr (AH) ah = lane_sum(ah, L);
    }

    __device__ __noinline__ double kernel_g_of(const Geo<DIM>& g) const {
        const KConst kx = make_kconst<DIM>(skf, hi);
        return kernel_g(skf, kx, g.r * kx.hinv, g.rinv);
    }

    // SPH = 1 (internalForce.f90:199-221) and SPH = 3 (:277-322) for a fluid
    // target, without the 1 / rho_i that the epilogue applies:
    //   ap += sum_j (T_j - P_j) V_j dW           (1)  or (T_j - 2 p*) V_j dW  (3)
    //   sw += sum_j V_j dW
    //   ein += (P_i + P_j) V_j dv.dW             (1)  or 4 p* V_j (v_i - v*).dW (3)
    __device__ __forceinline__ void internal_sch(int j, const Geo<DIM>& g, double gf, const double4& vj) {
        const double4 ej = d.eh[j];
        const double vg = ej.w * gf;   // V_j dW = (V_j g) dx
        const double Pj = d.pa4[j].y;
        const double* Tj = d.tt + (size_t)j * DIM * DIM;
        double ps = 0.0, dot = 0.0;
        if constexpr (SCH == 1) {
#pragma unroll
            for (int a = 0; a < DIM; ++a) dot = fma(g.dx[a], vi[a] - cmp(vj, a), dot);
        } else {
            // e = (x_j - x_i) / |x_j - x_i|; the Riemann state of the pair
            double e[DIM], vl = 0.0, vr = 0.0;
#pragma unroll
            for (int a = 0; a < DIM; ++a) {
                e[a] = -g.dx[a] * g.rinv;
                vl = fma(vi[a], e[a], vl);
                vr = fma(cmp(vj, a), e[a], vr);
            }
            const double Zl = rhoi * ci, Zr = vj.w * ej.z;
            const double iz = 1.0 / (Zl + Zr);
            const double vij = (Zl * vl + Zr * vr + (Pi - Pj)) * iz;
            ps = (Zl * Pj + Zr * Pi + (Zl * Zr) * (vl - vr)) * iz;
            const double vm = 0.5 * (vl + vr);
#pragma unroll
            for (int a = 0; a < DIM; ++a) {
                const double vs = vij * e[a] + (0.5 * (vi[a] + cmp(vj, a)) - vm * e[a]);
                dot = fma(vi[a] - vs, g.dx[a], dot);
            }
        }
        const double pw = SCH == 1 ? -Pj : -2.0 * ps;
#pragma unroll
        for (int a = 0; a < DIM; ++a) {
            const double wa = vg * g.dx[a];
            double t = fma(pw, wa, ap[a]);
#pragma unroll
            for (int b = 0; b < DIM; ++b) t = fma(Tj[b * DIM + a], vg * g.dx[b], t);
            ap[a] = t;
            sw[a] += wa;
        }
        ein = fma(SCH == 1 ? Pi + Pj : 4.0 * ps, vg * dot, ein);
    }
};

// SPH = 3 continuity (con_density_riemann, density.f90:110-148), before
// pass A: the pressure and sound speed are those of the previous EOS (or of
// the upload), as in the reference, where it runs before internal_force.
// drho_i = 2 rho_i sum_j V_j (v_i - v*) . dW_ij with Z_l = rho_i c_j (the
// reference takes the neighbour's sound speed on both sides), Z_r = rho_j c_j.
template <int DIM>
struct PhysR {
    const Dev& d;
    double xi[3], vi[3], rhoi, Pi;
    KConst kc;
    int skf;
    bool raw_walls;   // the instance's first step: walls as uploaded
    double acc = 0.0;
    __device__ PhysR(const Dev& dd, const double4& x, const double4& v, double h, double P, bool first, int i)
        : d(dd) {
        xi[0] = x.x; xi[1] = x.y; xi[2] = x.z;
        vi[0] = v.x; vi[1] = v.y; vi[2] = v.z;
        rhoi = v.w; Pi = P;
        skf = d.skf;
        kc = kconst_of<DIM>(d, i, skf, h);
        raw_walls = first && d.wraw != nullptr;
    }
    __device__ __forceinline__ void pair(int j) {
        const double4 xj = d.xm[j], vj = d.vr[j];
        double4 ej = d.eh[j];
        const Geo<DIM> g = geo<DIM>(xi, xj);
        const double gf = skf == 1 ? cubic_g_r(kc, g.r, g.rinv) : kernel_g(skf, kc, g.r * kc.hinv, g.rinv);
        double Pj;
        if (j < d.wall_off) {
            Pj = d.pold[j];
        } else if (raw_walls) {
            const double2 w = d.wraw[j];
            Pj = w.x;
            ej.z = w.y;
        } else {
            Pj = d.pa4[j].y;
        }
        double e[DIM], vl = 0.0, vr = 0.0;
#pragma unroll
        for (int a = 0; a < DIM; ++a) {
            e[a] = -g.dx[a] * g.rinv;
            vl = fma(vi[a], e[a], vl);
            vr = fma(cmp(vj, a), e[a], vr);
        }
        const double Zl = rhoi * ej.z, Zr = vj.w * ej.z;
        const double vij = (Zl * vl + Zr * vr + (Pi - Pj)) / (Zl + Zr);
        const double vm = 0.5 * (vl + vr);
        double dot = 0.0;
#pragma unroll
        for (int a = 0; a < DIM; ++a) {
            const double vs = vij * e[a] + (0.5 * (vi[a] + cmp(vj, a)) - vm * e[a]);
            dot = fma(vi[a] - vs, g.dx[a], dot);
        }
        acc = fma(ej.w * gf, dot, acc);
    }
};

template <int DIM>
__global__ void __launch_bounds__(TPB, 4) pass_r_kernel(const Dev d) {
    constexpr int K = ListLen<DIM>::K;
    extern __shared__ uint32_t smem[];
    uint32_t* lst = smem + (threadIdx.x >> 5) * ListLen<DIM>::SLOT;
    const int i = blockIdx.x * TPB + threadIdx.x;
    const bool valid = i < d.n_real;
    const int ii = valid ? i : 0;
    const double4 xm = d.xm[ii];
    const double4 vr = d.vr[ii];
    const double4 eh = d.eh[ii];
    const int4 meta = d.meta[ii];
    Target<DIM> t = make_target<DIM>(d, ii, xm, eh.y);
    PhysR<DIM> ph(d, xm, vr, eh.y, d.pold[ii], inst_of(d, ii).step == 0, ii);
    walk_lane<DIM, K>(d, t, valid && meta.w != -1, ph, lst, ExactAccept<DIM>{d, t});
    if (!valid) return;
    d.dvr[i].w = 2.0 * vr.w * ph.acc;
}

// pass B pair physics in double-float (fluid targets, cubic spline): the
// sums of PhysB (internal force, AV, energy); the external pair terms stay
// FP64 (the exact distance of the reference, behind the FP32 reach test).
// finalize() leaves the sums as doubles for the FP64 epilogue.
template <int DIM>
struct PhysBd {
    const Dev& d;
    uint32_t terms;
    DF xi[3], vi[3], rhoi, hi, ci, Pid;
    double xa[3], hid, cid, Pi;
    int typei;
    bool solid_i = false;
    double alpha, beta;
    DF alphad, betad, psid, psi_q, alpha_h;
    KConstD kc;
    const Inst* I;
    DFAcc apd[DIM], swd[DIM], eind, aavd[DIM], eavd;
    double ap[DIM], sw[DIM], ein, aav[DIM], eav, aex[DIM], aas[DIM];
    __device__ PhysBd(const Dev& dd, uint32_t tm, const double4& x, const double4& v, const double4& e, double P,
                      int type, const Inst* inst, int i) : d(dd), terms(tm), I(inst) {
        xa[0] = x.x; xa[1] = x.y; xa[2] = x.z;
        hid = e.y; cid = e.z; Pi = P; typei = type;
        rhoi = df_from(v.w); hi = df_from(e.y); ci = df_from(e.z); Pid = df_from(P);
        alpha = type > 100 ? d.av_alpha_solid : d.av_alpha;
        beta = type > 100 ? d.av_beta_solid : d.av_beta;
        alphad = df_from(alpha); betad = df_from(beta); psid = df_from(d.av_psi);
        psi_q = df_from(0.25 * (d.av_psi * d.av_psi));
        alpha_h = df_from(-0.5 * alpha);
        kc = make_kconst_d(kconst_of<DIM>(d, i, 1, e.y));
#pragma unroll
        for (int a = 0; a < DIM; ++a) {
            aex[a] = 0.0;
            aas[a] = 0.0;
        }
        if ((terms & SPH_TERM_EXTERNAL) && (d.flags & SPH_F_GRAVITY) &&
            !((d.flags & SPH_F_GRAVITY_SKIP_SOLIDS) && type > 100))
            aex[DIM - 1] = d.gravity;
    }
    __device__ __forceinline__ void target(int i) {
        const float4 a0 = d.pd0[i], a1 = d.pd1[i], v0 = d.vd0[i], v1 = d.vd1[i];
        xi[0] = DF{a0.x, a1.x}; xi[1] = DF{a0.y, a1.y}; xi[2] = DF{a0.z, a1.z};
        vi[0] = DF{v0.x, v1.x}; vi[1] = DF{v0.y, v1.y}; vi[2] = DF{v0.z, v1.z};
    }
    __device__ __forceinline__ void pair(int j) {
        const float4 a0 = d.pd0[j], a1 = d.pd1[j], v0 = d.vd0[j], v1 = d.vd1[j];
        const GeoD<DIM> g = geo_d<DIM>(xi, a0, a1, kc);
        const DF mg = df_mul(DF{a0.w, a1.w}, g.gf);
        const DF vj[3] = {DF{v0.x, v1.x}, DF{v0.y, v1.y}, DF{v0.z, v1.z}};
        DF w[DIM], dv[DIM], xv = DF{0.0f, 0.0f};
#pragma unroll
        for (int a = 0; a < DIM; ++a) {
            w[a] = df_mul(mg, g.dx[a]);
            dv[a] = df_sub(vi[a], vj[a]);
            xv = df_fma(g.dx[a], dv[a], xv);
        }
        const DF dvw = df_mul(mg, xv);
        if (terms & SPH_TERM_INTERNAL) {
            const float4 e1 = d.ed1[j];
            const DF Pj = DF{e1.z, e1.w};
            const float2* Tj = d.ttd + (size_t)j * DIM * DIM;
#pragma unroll
            for (int a = 0; a < DIM; ++a) {
#pragma unroll
                for (int b = 0; b < DIM; ++b) {   // (T_j - P_j I) . m_j dW
                    const float2 T = Tj[b * DIM + a];
                    apd[a].add_prod(DF{T.x, T.y}, w[b]);
                }
                swd[a].add(w[a]);
            }
            eind.add_prod(df_add(Pid, Pj), dvw);
        }
        if ((terms & SPH_TERM_ARTI_VISC) && xv.hi < 0.0f) {
            const float4 e0 = d.ed0[j], e1 = d.ed1[j];
            const DF hj = DF{e0.z, e0.w}, cj = DF{e1.x, e1.y}, rhoj = DF{v0.w, v1.w};
            DF PI;
            if (beta == 0.0) {
                const DF sh = df_add(hi, hj);
                const DF D = df_fma(df_mul(psi_q, sh), sh, g.dr);
                PI = df_mul(df_mul(df_mul(alpha_h, df_add(ci, cj)), df_mul(sh, xv)), df_rcp(df_mul(D, df_add(rhoi, rhoj))));
            } else {
                const DF hij = df_mul_f(df_add(hi, hj), 0.5f);
                const DF rij = df_mul_f(df_add(rhoi, rhoj), 0.5f);
                const DF cij = df_mul_f(df_add(ci, cj), 0.5f);
                const DF ph = df_mul(psid, hij);
                const DF D = df_fma(ph, ph, g.dr);
                const DF hx = df_mul(hij, xv);
                const DF num = df_mul(hx, df_sub(df_mul(betad, hx), df_mul(df_mul(alphad, cij), D)));
                PI = df_mul(num, df_rcp(df_mul(df_mul(D, D), rij)));
            }
#pragma unroll
            for (int a = 0; a < DIM; ++a) aavd[a].add_prod(df_neg(PI), w[a]);
            eavd.add_prod(PI, dvw);
        }
        if (terms & SPH_TERM_EXTERNAL) {
            const int tj = d.meta[j].x;
            if (typei > 0 && (tj < 0 || tj != typei) &&
                g.dr.hi <= ext_reach2(*I, tj < 0, (float)hid, d.ed0[j].z))
                external_pair<DIM>(d, *I, xa, hid, cid, typei, j, tj, d.xm[j], aex);
        }
    }
    __device__ __forceinline__ void finalize() {
#pragma unroll
        for (int a = 0; a < DIM; ++a) {
            ap[a] = apd[a].to_double();
            sw[a] = swd[a].to_double();
            aav[a] = aavd[a].to_double();
        }
        ein = eind.to_double();
        eav = eavd.to_double();
    }
};

template <int DIM, bool SOLID, bool KGC = false, bool DFM = false, int SCH = 2, bool AH = false, bool LS = false>
__global__ void __launch_bounds__(TPB, 4) pass_b_kernel(const Dev d, uint32_t terms, int assemble) {
    static_assert(!LS || (!KGC && !DFM), "lanes per target: the plain FP64 form");
    constexpr int K = ListLen<DIM, true, true>::K;
    constexpr int D2 = DIM * DIM;
    extern __shared__ uint32_t smem[];
    uint32_t* lst = smem + (threadIdx.x >> 5) * ListLen<DIM, true, true>::SLOT;
    float4* tile = reinterpret_cast<float4*>(lst + K * 32);
    const int gt = blockIdx.x * TPB + threadIdx.x;
    const int lsh = LS ? d.lane_shift : 0;
    const int i = gt >> lsh;
    const bool valid = i < d.n_real;
    const int ii = valid ? i : 0;
    const double4 xm = d.xm[ii];
    const double4 vr = d.vr[ii];
    const double4 eh = d.eh[ii];
    const int4 meta = d.meta[ii];
    const double4 pa = d.pa4[ii];
    Target<DIM> t = make_target<DIM>(d, ii, xm, eh.y);
    using PB = std::conditional_t<DFM, PhysBd<DIM>, PhysB<DIM, SOLID, KGC, SCH, AH>>;
    PB ph(d, terms, xm, vr, eh, SCH == 2 ? pa.x : pa.y, meta.x, &inst_of(d, ii), ii);
    if constexpr (KGC) ph.kf = d.kgc + (size_t)ii * KGC_STRIDE;
    if constexpr (AH && !DFM) {
        ph.qi = (0.1 * eh.y) * eh.z + (eh.y * eh.y) * (fabs(pa.z) - pa.z);
        ph.ei = eh.x;
    }
    if constexpr (DFM) ph.target(ii);
    if constexpr (SOLID && DIM == 2 && !DFM) {
        if (terms & SPH_TERM_ARTI_STRESS) {
            ph.wd = kernel_w(d.skf, ph.kc, inst_of(d, ii).as_dp * ph.kc.hinv);
            ph.Ri = d.ras[ii];
        }
    }
    if constexpr (DFM) {
        walk_tiled<DIM, K, PB, true>(d, t, valid && meta.w != -1, ph, lst, tile, 0.0f, SplitDF(d, ii));
        ph.finalize();
    } else if constexpr (LS) {
        const LaneShare share{gt & ((1 << lsh) - 1), (1 << lsh) - 1};
        ph.lane_start(share.sub);
        walk_tiled<DIM, K, PB, true, SplitFP64, LaneShare>(d, t, valid && meta.w != -1, ph, lst, tile, 0.0f,
                                                           SplitFP64(d, vr), share);
        ph.lane_sums(1 << lsh);
        if (share.sub != 0) return;
    } else {
        walk_tiled<DIM, K, PB, true>(d, t, valid && meta.w != -1, ph, lst, tile, 0.0f, SplitFP64(d, vr));
    }
    if (!valid) return;

    double a[DIM];
    double de = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) a[k] = 0.0;
    if (SCH != 2 && (terms & SPH_TERM_INTERNAL)) {
        // T_i (- P_i under SPH = 1) times sum_j V_j dW, all over rho_i; a
        // solid target gets none (internalForce.f90:222, 323)
        de = d.tds[i];
        if (!ph.solid_i) {
            const double* Ti = d.tt + (size_t)i * D2;
            const double ir = 1.0 / vr.w;
#pragma unroll
            for (int r = 0; r < DIM; ++r) {
                double s = SCH == 1 ? fma(-ph.Pi, ph.sw[r], ph.ap[r]) : ph.ap[r];
#pragma unroll
                for (int b = 0; b < DIM; ++b) s = fma(Ti[b * DIM + r], ph.sw[b], s);
                a[r] = s * ir;
            }
            de += 0.5 * (ph.ein * ir);
        }
    } else if (terms & SPH_TERM_INTERNAL) {
        // T_i - P_i I (resp. sigma_i / rho_i^2) times sum_j m_j dW
        const double* Ti = (SOLID && ph.solid_i) ? d.sig + (size_t)i * D2 : d.tt + (size_t)i * D2;
#pragma unroll
        for (int r = 0; r < DIM; ++r) {
            double s = ph.ap[r];
#pragma unroll
            for (int b = 0; b < DIM; ++b) s = fma(Ti[b * DIM + r], ph.sw[b], s);
            a[r] = s;
        }
        de = d.tds[i] + 0.5 * ph.ein;  // internalForce.f90:332-334
    }
    // Delta%Velocity = in + av + ex + as (singleStep.f90:139-142)
    if (terms & SPH_TERM_ARTI_VISC) {
#pragma unroll
        for (int k = 0; k < DIM; ++k) a[k] += ph.aav[k];
        de += 0.5 * ph.eav;
    }
    if constexpr (AH && !DFM) {   // Delta%Energy = in + av + ah (singleStep.f90:141)
        if (terms & SPH_TERM_ARTI_HEAT) de += ph.ah;
    }
    if (terms & SPH_TERM_EXTERNAL) {
#pragma unroll
        for (int k = 0; k < DIM; ++k) a[k] += ph.aex[k];
    }
    if (terms & SPH_TERM_ARTI_STRESS) {
#pragma unroll
        for (int k = 0; k < DIM; ++k) a[k] += ph.aas[k];
    }
    if (assemble && meta.y == 1) {  // fixedBoundary
#pragma unroll
        for (int k = 0; k < DIM; ++k) a[k] = 0.0;
    }
    double4 out = d.dvr[i];
    out.x = a[0];
    out.y = DIM > 1 ? a[1] : 0.0;
    out.z = DIM > 2 ? a[2] : 0.0;
    d.dvr[i] = out;
    d.dedt[i] = de;
}


// ===========================================================================
// Mixed precision (SPH_PREC_MIXED): FP32 kernel weights, EOS and pair forces
// with Kahan-compensated sums, on positions relative to each particle's cell
// origin (FP32 rounding of x - origin, about 1e-9 m at 4 mm cells, instead of
// the absolute position).  Positions, velocities and the leap-frog update
// stay FP64; so do the Courant reduction and the external-force pair terms.
// ===========================================================================
__device__ __forceinline__ float p4f(float a) { float a2 = a * a; return a2 * a2; }
__device__ __forceinline__ float p5f(float a) { float a2 = a * a; return (a2 * a2) * a; }

__device__ __forceinline__ float kernel_g_f(int skf, const KConstF& k, float q, float rinv) {
    if (skf == 1) {
        const float t = 2.0f - q;
        return q < 1.0f ? fmaf(k.A2, q, k.A1) : (k.A3 * (t * t)) * rinv;
    } else if (skf == 2) {
        return q < 3.0f ? (k.factor * __expf(-q * q)) * k.A1 : 0.0f;
    } else {
        const float f = k.factor;
        if (q < 1.0f) return (f * ((-120.0f + 120.0f * q) - 50.0f * (q * q))) * (k.hinv * k.hinv);
        if (q < 2.0f) return ((f * (-5.0f * p4f(3.0f - q) + 30.0f * p4f(2.0f - q))) * k.hinv) * rinv;
        if (q <= 3.0f) return ((f * (-5.0f * p4f(3.0f - q))) * k.hinv) * rinv;
        return 0.0f;
    }
}

__device__ __forceinline__ float kernel_w_f(int skf, const KConstF& k, float q) {
    if (skf == 1) {
        if (q < 1.0f) return k.factor * ((2.0f / 3.0f - q * q) + (q * q * q) * 0.5f);
        if (q <= 2.0f) { const float t = 2.0f - q; return k.factor * (1.0f / 6.0f) * (t * t * t); }
        return 0.0f;
    } else if (skf == 2) {
        return q < 3.0f ? k.factor * __expf(-q * q) : 0.0f;
    } else {
        const float f = k.factor;
        if (q < 1.0f) return f * ((p5f(3.0f - q) - 6.0f * p5f(2.0f - q)) + 15.0f * p5f(1.0f - q));
        if (q < 2.0f) return f * (p5f(3.0f - q) - 6.0f * p5f(2.0f - q));
        if (q <= 3.0f) return f * p5f(3.0f - q);
        return 0.0f;
    }
}

__device__ __forceinline__ float pow_int_or_real_f(float x, float e) {
    if (e == 7.0f) { const float x2 = x * x, x4 = x2 * x2; return (x4 * x2) * x; }
    if (e == 12.0f) { const float x4 = p4f(x); return (x4 * x4) * x4; }
    if (e == 6.0f) { const float x2 = x * x; return (x2 * x2) * x2; }
    if (e == 4.0f) return p4f(x);
    if (e == 2.0f) return x * x;
    return powf(x, e);
}

__device__ __forceinline__ void fluid_eos_f(const DevMaterial* m, float rho, float e, float& p, float& c) {
    if (!m) return;
    switch (m->eos) {
    case SPH_EOS_GAS: { const float g = m->gamma_f; p = (g - 1.0f) * rho * e; c = sqrtf(g * p / rho); } break;
    case SPH_EOS_TAIT: p = m->tait_b_f * (pow_int_or_real_f(rho / m->rho0_f, m->gamma_f) - 1.0f); break;
    case SPH_EOS_MORRIS: c = 0.01f; p = (c * c) * rho; break;
    case SPH_EOS_LINEAR: p = m->k_rho0_f * (rho - m->rho0_f); break;
    default: break;
    }
}

__device__ __forceinline__ void solid_eos_f(const DevMaterial* m, float rho, float e, float& p) {
    if (!m) return;
    if (m->eos == SPH_EOS_MG_SOLID) {
        const float r0 = m->rho0_f, cs = m->mg_cs_f, sl = m->mg_s_f, G = m->gamma_f;
        const float mu = rho / r0 - 1.0f;
        const float p1 = r0 * (cs * cs);
        const float p2 = p1 * (1.0f + 2.0f * (sl - 1.0f));
        const float p3 = p1 * (2.0f * (sl - 1.0f) + 3.0f * ((sl - 1.0f) * (sl - 1.0f)));
        const float pH = mu > 0.0f ? (p1 * mu + p2 * (mu * mu)) + p3 * ((mu * mu) * mu) : p1 * mu;
        p = (1.0f - (0.5f * G) * mu) * pH + (G * rho) * e;
    } else if (m->eos == SPH_EOS_LINEAR) {
        p = m->k_rho0_f * (rho - m->rho0_f);
    }
}

template <int DIM>
struct TargetM {
    int i;
    float xr[3];
    uint32_t code5;   // the cell code plus 0x555 (rel_dx)
    float reach2;
    float cs;
};

template <int DIM>
__device__ __forceinline__ TargetM<DIM> make_target_m(const Dev& d, int i, double h) {
    TargetM<DIM> t;
    t.i = i;
    const float4 p = d.pr4[i];
    t.xr[0] = p.x; t.xr[1] = p.y; t.xr[2] = p.z;
    t.code5 = (uint32_t)__float_as_int(p.w) + 0x555u;
    if (const KRef* r = kref_for(d, i, d.skf, h)) {
        t.reach2 = r->reach2f;
    } else {
        const float reach = (float)(h * (double)d.scale_k);
        t.reach2 = reach * reach;
    }
    t.cs = inst_of(d, i).grid.cs_f;
    return t;
}

template <int DIM>
__device__ __forceinline__ void rel_dx(const TargetM<DIM>& t, const float4& pj, float* dx) {
    // per 4-bit field (c_i + 5 - c_j) lies in 2..8, so one subtraction keeps
    // the three axes apart; & 3 leaves k = c_i - c_j + 1 in {0, 1, 2}, and
    // 2^23 + k - (2^23 + 1) is k - 1 as a float (no int-to-float conversion,
    // which would issue on the FP64 pipe).  (k - 1) cs is exact, so the fma
    // rounds like (x_i - x_j) + (c_i - c_j) cs.
    const uint32_t k = (t.code5 - (uint32_t)__float_as_int(pj.w)) & 0x333u;
    const float f0 = __uint_as_float(0x4B000000u | (k & 3u)) - 8388609.0f;
    const float f1 = __uint_as_float(0x4B000000u | ((k >> 4) & 3u)) - 8388609.0f;
    dx[0] = fmaf(f0, t.cs, t.xr[0] - pj.x);
    dx[1] = fmaf(f1, t.cs, t.xr[1] - pj.y);
    if constexpr (DIM == 3) {
        const float f2 = __uint_as_float(0x4B000000u | (k >> 8)) - 8388609.0f;
        dx[2] = fmaf(f2, t.cs, t.xr[2] - pj.z);
    } else {
        dx[2] = 0.0f;
    }
}

// The mixed path's neighbour test (walk_tiled): r^2 < (scale_k h)^2 on the
// FP32 positions relative to the grid origin (pairs within FP32 rounding of
// the cut-off may differ from the FP64 set; their kernel weight is ~0).

template <int DIM>
struct PhysAm {
    const Dev& d;
    const TargetM<DIM>& t;
    float vi[3];
    KConstF kc;
    int skf;
    // The velocity gradient G[a][b] and sum_j V_j dx.dW as packed Kahan pairs:
    // 3-D (G00,G01) (G10,G11) (G20,G21) (G02,G12) (G22,sdx); 2-D (G00,G01)
    // (G10,G11) and sdx alone.
    KSum2 Gp[DIM == 3 ? 5 : 2];
    KSum sdx2;
    int nn = 0;
    bool xsph;
    float rhoi;
    KSum axs[DIM];
    __device__ __forceinline__ double Gv(int a, int b) const {
        if (DIM == 2 || b < 2) return b == 0 ? Gp[a].x() : Gp[a].y();
        return a == 0 ? Gp[DIM == 3 ? 3 : 0].x() : (a == 1 ? Gp[DIM == 3 ? 3 : 0].y() : Gp[DIM == 3 ? 4 : 0].x());
    }
    __device__ __forceinline__ float Gvf(int a, int b) const {   // Gv rounded to FP32
        if (DIM == 2 || b < 2) return b == 0 ? Gp[a].xf() : Gp[a].yf();
        return a == 0 ? Gp[DIM == 3 ? 3 : 0].xf() : (a == 1 ? Gp[DIM == 3 ? 3 : 0].yf() : Gp[DIM == 3 ? 4 : 0].xf());
    }
    __device__ __forceinline__ double sdxv() const { return DIM == 3 ? Gp[DIM == 3 ? 4 : 0].y() : sdx2.value(); }
    __device__ PhysAm(const Dev& dd, const TargetM<DIM>& tt, double h) : d(dd), t(tt) {
        // the target's FP32 mirror: the conversions of its v and rho
        const float4 v = d.vf4[t.i];
        vi[0] = v.x; vi[1] = v.y; vi[2] = v.z;
        rhoi = v.w;
        xsph = d.flags & SPH_F_AVER_VELOCITY;
        skf = d.skf;
        kc = kconst_f_of<DIM>(d, t.i, skf, h);
    }
    __device__ __forceinline__ void pair(int j) {
        const float4 pj = d.pr4[j];
        const float4 vj = d.vf4[j];
        const float Vj = d.ef4[j].z;
        float dx[3];
        rel_dx<DIM>(t, pj, dx);
        float dr = dx[0] * dx[0] + dx[1] * dx[1];
        if (DIM == 3) dr += dx[2] * dx[2];
        const float rinv = dr > 0.0f ? rsqrtf(dr) : 0.0f;
        const float q = (dr * rinv) * kc.hinv;
        const float g = kernel_g_f(skf, kc, q, rinv);
        const float vjv[3] = {vj.x, vj.y, vj.z};
        float u[DIM];
#pragma unroll
        for (int a = 0; a < DIM; ++a) u[a] = (Vj * (vjv[a] - vi[a])) * g;
        const float2 dx01 = make_float2(dx[0], dx[1]);
#pragma unroll
        for (int a = 0; a < DIM; ++a) Gp[a].add_prod(make_float2(u[a], u[a]), dx01);
        if constexpr (DIM == 3) {
            Gp[3].add_prod(make_float2(u[0], u[1]), make_float2(dx[2], dx[2]));
            Gp[4].add_prod(make_float2(u[2], Vj), make_float2(dx[2], g * dr));
        } else {
            sdx2.add(Vj * (g * dr));
        }
        ++nn;
        if (xsph) {
            const float W = kernel_w_f(skf, kc, q);
            const float f = ((d.xsph_eps2_f * d.ef4[j].w) / (rhoi + vj.w)) * W;
#pragma unroll
            for (int a = 0; a < DIM; ++a) axs[a].add(f * (vi[a] - vjv[a]));
        }
    }
};

template <int DIM, bool SOLID, int K>
__device__ __forceinline__ void pass_a_mixed_targets(const Dev& d, int i, int want_strain, uint32_t* lst,
                                                     float4* tile) {
    constexpr int D2 = DIM * DIM;
    const bool valid = i < d.n_real;
    const int ii = valid ? i : 0;
    const double4 xm = d.xm[ii];
    const double4 vr = d.vr[ii];
    const double4 eh = d.eh[ii];
    const int4 meta = d.meta[ii];
    const Target<DIM> tc = make_target<DIM>(d, ii, xm, eh.y);
    const TargetM<DIM> t = make_target_m<DIM>(d, ii, eh.y);
    PhysAm<DIM> ph(d, t, eh.y);
    walk_tiled<DIM, K>(d, tc, valid && meta.w != -1, ph, lst, tile, t.reach2);
    if (!valid) return;

    // FP32 values from the mirrors and the FP32 copies of the material
    const float4 ef = d.ef4[i];
    const float rho = ph.rhoi;
    const int type = meta.x;
    const bool visc = d.flags & SPH_F_VISCOSITY;
    const DevMaterial* m = material_of(d, inst_of(d, i), type);
    const float eta = (visc && m) ? m->eta_f : 0.0f;
    float G[DIM][DIM];
#pragma unroll
    for (int a = 0; a < DIM; ++a)
#pragma unroll
        for (int b = 0; b < DIM; ++b) G[a][b] = ph.Gvf(a, b);
    float divv = 0.0f;
#pragma unroll
    for (int a = 0; a < DIM; ++a) divv += G[a][a];
    const double divx = -ph.sdxv();
    float p = (float)d.pa4[i].y, c = ef.y;
    float edot[DIM][DIM];
    float tds = 0.0f;
    const float rho2 = rho * rho;
    const bool solid = SOLID && is_solid_type(type);
    if (!solid) {
#pragma unroll
        for (int a = 0; a < DIM; ++a)
#pragma unroll
            for (int b = 0; b < DIM; ++b)
                edot[a][b] = visc ? 2.0f * G[a][b] - (a == b ? (2.0f / 3.0f) * divv : 0.0f) : 0.0f;
        if (visc) {
            float s = 0.0f;
#pragma unroll
            for (int b = 0; b < DIM; ++b)
#pragma unroll
                for (int a = 0; a < DIM; ++a) s += edot[a][b] * edot[a][b];
            tds = 0.5f * eta / rho * s;
        }
        fluid_eos_f(m, rho, (float)eh.x, p, c);
        if (SOLID) {
#pragma unroll
            for (int k = 0; k < D2; ++k) d.sf[(size_t)i * tf_stride_of(DIM) + k] = 0.0f;
            if (DIM == 2) d.rf4[i] = make_float4(0, 0, 0, 0);
        }
    } else {
        float rot[DIM][DIM];
#pragma unroll
        for (int a = 0; a < DIM; ++a)
#pragma unroll
            for (int b = 0; b < DIM; ++b) {
                edot[a][b] = visc ? 0.5f * (G[a][b] + G[b][a]) : 0.0f;
                rot[a][b] = visc ? 0.5f * (G[a][b] - G[b][a]) : 0.0f;
            }
        float tr = 0.0f;
#pragma unroll
        for (int a = 0; a < DIM; ++a) tr += edot[a][a];
        tr = tr / 3.0f;
        float eb[DIM][DIM], S[DIM][DIM];
        const double* sh = d.shear + (size_t)i * D2;
#pragma unroll
        for (int b = 0; b < DIM; ++b)
#pragma unroll
            for (int a = 0; a < DIM; ++a) {
                S[a][b] = (float)sh[b * DIM + a];
                eb[a][b] = edot[a][b] - (a == b ? tr : 0.0f);
            }
        float s = 0.0f;
#pragma unroll
        for (int b = 0; b < DIM; ++b)
#pragma unroll
            for (int a = 0; a < DIM; ++a) s += S[a][b] * eb[a][b];
        tds = s / rho;
        solid_eos_f(m, rho, (float)eh.x, p);
        const float G2 = 2.0f * eta;
        double* ds = d.dsdt + (size_t)i * D2;
        float* sg = d.sf + (size_t)i * tf_stride_of(DIM);
        const float irho2 = 1.0f / rho2;
#pragma unroll
        for (int a = 0; a < DIM; ++a)
#pragma unroll
            for (int b = 0; b < DIM; ++b) {
                float v = G2 * eb[a][b];
#pragma unroll
                for (int k = 0; k < DIM; ++k) v += S[a][k] * rot[b][k] + S[b][k] * rot[a][k];
                ds[b * DIM + a] = (double)v;
                sg[b * DIM + a] = (S[a][b] - (a == b ? p : 0.0f)) * irho2;
            }
        if (DIM == 2) {
            float4 R = make_float4(0, 0, 0, 0);
            if (type >= 100) {
                const float s11 = S[0][0] - p, s22 = S[1][1] - p, s12 = S[0][1], s21 = S[1][0];
                const float aux = s11 - s22;
                const float th = aux == 0.0f ? 0.5f * 3.14159265358979f : 0.5f * atanf((s12 + s21) / aux);
                float sn, cs;
                sincosf(th, &sn, &cs);
                const float ps0 = (cs * cs) * s11 + (sn * sn) * s22 + 2.0f * sn * cs * s12;
                const float ps1 = (sn * sn) * s11 + (cs * cs) * s22 - 2.0f * sn * cs * s12;
                const float eps = d.as_eps_f;
                const float T0 = ps0 > 0.0f ? -(eps * ps0 / rho2) : 0.0f;
                const float T1 = ps1 > 0.0f ? -(eps * ps1 / rho2) : 0.0f;
                R.x = (cs * cs) * T0 + (sn * sn) * T1;
                R.y = (sn * sn) * T0 + (cs * cs) * T1;
                R.z = sn * cs * (T0 - T1);
            }
            d.rf4[i] = R;
        }
    }
    float* tf = d.tf + (size_t)i * tf_stride_of(DIM);
    const bool drop_tt = solid && (d.flags & SPH_F_FSI_FLUID_VISCOUS);
#pragma unroll
    for (int b = 0; b < DIM; ++b)
#pragma unroll
        for (int a = 0; a < DIM; ++a) tf[b * DIM + a] = drop_tt ? 0.0f : eta * edot[a][b] / rho2;
    if (want_strain) {
        double* st = d.strain + (size_t)i * D2;
#pragma unroll
        for (int b = 0; b < DIM; ++b)
#pragma unroll
            for (int a = 0; a < DIM; ++a) st[b * DIM + a] = (double)edot[a][b];
    }
    const float P = p / rho2;
    const double divvd = (double)divv;
    d.pf4[i] = make_float4(P, p, __int_as_float(type), 0.0f);
    d.pa4[i] = make_double4((double)P, (double)p, divvd, divx);
    d.tds[i] = (double)tds;
    if (c != ef.y) { d.eh[i].z = (double)c; d.ef4[i].y = c; }
    if (d.dxp) d.dxp[i] = divx;
    if (!(d.flags & SPH_F_SUM_DENSITY)) d.dvr[i].w = -vr.w * divvd;
    else d.dvr[i].w = 0.0;
    if (ph.xsph) {
        double v[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int a = 0; a < DIM; ++a) v[a] = meta.y == 1 ? 0.0 : -ph.axs[a].value();
        d.aver[i] = make_double4(v[0], v[1], v[2], 0.0);
    }
    d.nneigh[i] = ph.nn;
}

// One tile of blockDim.x targets per block, or (PERSIST, SPH_OPT_PERSISTENT)
// only as many blocks as are resident, each striding over the tiles.  The
// persistent form is a separate instantiation, so that the loop does not
// change the code of the default one.
template <int DIM, bool SOLID, int K, bool PERSIST>
__global__ void __launch_bounds__(MAX_TILE_TPB, DIM == 2 ? MIXED_A_MINB_2D : 4) pass_a_mixed_kernel(const Dev d, int want_strain) {
    extern __shared__ uint32_t smem[];
    uint32_t* lst = smem + (threadIdx.x >> 5) * tiled_slot(K);
    float4* tile = reinterpret_cast<float4*>(lst + K * 32);
    if constexpr (PERSIST) {
        for (int base = blockIdx.x * blockDim.x; base < d.n_real; base += gridDim.x * blockDim.x)
            pass_a_mixed_targets<DIM, SOLID, K>(d, base + (int)threadIdx.x, want_strain, lst, tile);
    } else {
        pass_a_mixed_targets<DIM, SOLID, K>(d, (int)(blockIdx.x * blockDim.x + threadIdx.x), want_strain, lst, tile);
    }
}

// Summation density in FP32 (kernel weights, Kahan sums); the self term and
// the normalisation are applied in FP64.
template <int DIM>
struct PhysSm {
    const Dev& d;
    const TargetM<DIM>& t;
    KConstF kc;
    int skf;
    bool norm;
    KSum rho, wv;
    __device__ PhysSm(const Dev& dd, const TargetM<DIM>& tt, double h, bool nrm) : d(dd), t(tt), norm(nrm) {
        skf = d.skf;
        kc = kconst_f_of<DIM>(d, t.i, skf, h);
    }
    __device__ __forceinline__ void pair(int j) {
        const float4 pj = d.pr4[j];
        const float4 ej = d.ef4[j];
        float dx[3];
        rel_dx<DIM>(t, pj, dx);
        float dr = dx[0] * dx[0] + dx[1] * dx[1];
        if (DIM == 3) dr += dx[2] * dx[2];
        const float rinv = dr > 0.0f ? rsqrtf(dr) : 0.0f;
        const float w = kernel_w_f(skf, kc, (dr * rinv) * kc.hinv);
        rho.add(ej.w * w);
        if (norm) wv.add(ej.z * w);
    }
};

template <int DIM, int K>
__device__ __forceinline__ void pass_s_mixed_targets(const Dev& d, int i, uint32_t* lst, float4* tile) {
    const bool valid = i < d.n_real;
    const int ii = valid ? i : 0;
    const double4 xm = d.xm[ii];
    const double4 eh = d.eh[ii];
    const int4 meta = d.meta[ii];
    const bool norm = (d.flags & SPH_F_NORM_DENSITY) && d.dxp[ii] < 1.5;
    const Target<DIM> tc = make_target<DIM>(d, ii, xm, eh.y);
    const TargetM<DIM> t = make_target_m<DIM>(d, ii, eh.y);
    PhysSm<DIM> ph(d, t, eh.y, norm);
    walk_tiled<DIM, K>(d, tc, valid && meta.w != -1, ph, lst, tile, t.reach2);
    if (!valid) return;
    const double self = (double)kernel_w_f(ph.skf, ph.kc, 0.0f);
    double rho = xm.w * self + ph.rho.value();
    if (norm) rho = rho / (eh.w * self + ph.wv.value());
    d.rsum[i] = rho;
}

template <int DIM, int K, bool PERSIST>
__global__ void __launch_bounds__(MAX_TILE_TPB, DIM == 2 ? MIXED_A_MINB_2D : 4) pass_s_mixed_kernel(const Dev d) {
    extern __shared__ uint32_t smem[];
    uint32_t* lst = smem + (threadIdx.x >> 5) * tiled_slot(K);
    float4* tile = reinterpret_cast<float4*>(lst + K * 32);
    if constexpr (PERSIST) {
        for (int base = blockIdx.x * blockDim.x; base < d.n_real; base += gridDim.x * blockDim.x)
            pass_s_mixed_targets<DIM, K>(d, base + (int)threadIdx.x, lst, tile);
    } else {
        pass_s_mixed_targets<DIM, K>(d, (int)(blockIdx.x * blockDim.x + threadIdx.x), lst, tile);
    }
}

// The external pair terms of external_pair in FP32, for the mixed passes.
// Each term is continuous where its switch turns it on (zero force at r0, at
// pe = 1, at r = delta and at eta = 2), so the FP32 rounding of r moves a
// switch only across a margin where the force is about zero.
template <int DIM>
__device__ __forceinline__ void external_pair_f(const Dev& d, const Inst& I, const float* dx, float dr, float hi,
                                                float ci, int typei, int tj, float hj, KSum* aex) {
    const bool wallpair = typei > 0 && tj < 0;
    const bool phase = typei != tj && typei > 0 && tj > 0;
    if (!wallpair && !phase) return;
    const float r = sqrtf(dr);
    const float r2 = r * r;
    float f = 0.0f;
    if (wallpair && r < I.wall_r0_f) {
        const float t = I.wall_r0_f / r;
        f = d.wall_fs_f * (pow_int_or_real_f(t, d.wall_p1_f) - pow_int_or_real_f(t, d.wall_p2_f));
    }
    if (phase) {
        if (typei < 100 && tj < 100) {  // multiphase penalty
            const float pe = (hi + hj) / (2.0f * r);
            if (pe >= 1.0f) f = d.pen_factor_f * (pow_int_or_real_f(pe, d.pen_n1_f) - pow_int_or_real_f(pe, d.pen_n2_f));
        } else if (!(typei > 100 && tj > 100)) {  // fluid-solid contact
            const float eta = r / 0.75f / ((hi + hj) * 0.5f);
            float chi = 1.0f - r / I.ext_delta;
            if (chi < 0.0f || chi > 1.0f) chi = 0.0f;
            float fc;
            if (eta <= 0.0f || eta >= 2.0f) fc = 0.0f;
            else if (eta <= 2.0f / 3.0f) fc = 2.0f / 3.0f;
            else if (eta <= 1.0f) fc = 2.0f * eta - 1.5f * eta * eta;
            else fc = 0.5f * ((2.0f - eta) * (2.0f - eta));
            f = 0.01f * (ci * ci) * chi * fc;
        }
    }
    if (f != 0.0f) {
#pragma unroll
        for (int a = 0; a < DIM; ++a) aex[a].add(f * dx[a] / r2);
    }
}

// A neighbour's FP32 tensor row (tf or sf) as aligned float4 loads.
template <int DIM>
__device__ __forceinline__ void load_tensor_f(const float* base, int j, float* T) {
    const float4* r = reinterpret_cast<const float4*>(base + (size_t)j * tf_stride_of(DIM));
#pragma unroll
    for (int q = 0; q < tf_stride_of(DIM) / 4; ++q) {
        const float4 v = r[q];
        T[4 * q] = v.x; T[4 * q + 1] = v.y; T[4 * q + 2] = v.z; T[4 * q + 3] = v.w;
    }
}

template <int DIM, bool SOLID>
struct PhysBm {
    static constexpr bool early_entry = DIM == 3;   // see walk_tiled (2-D measured 0.7 % slower)
    const Dev& d;
    const TargetM<DIM>& t;
    uint32_t terms;
    float vi[3], hi, rhoi, ci, Pi;
    int typei;
    bool solid_i;
    float alpha, beta, psi;
    KConstF kc;
    int skf;
    float wd;
    float4 Ri;
    const Inst* I;
    // (ap[a], sw[a]) as packed Kahan pairs; the AV sums as (aav0, aav1) and,
    // in 3-D, (aav2, eav); in 2-D eav alone in the x of av2e
    KSum2 apsw[DIM];
    KSum ein;
    KSum2 av01;
    KSum2 av2e;
    KSum aas[DIM], aexp[DIM];
    double aex[DIM];
    __device__ __forceinline__ double apv(int a) const { return apsw[a].x(); }
    __device__ __forceinline__ double swv(int a) const { return apsw[a].y(); }
    __device__ __forceinline__ double aavv(int a) const {
        return a == 0 ? av01.x() : (a == 1 ? av01.y() : av2e.x());
    }
    __device__ __forceinline__ double eavv() const { return DIM == 3 ? av2e.y() : av2e.x(); }
    __device__ PhysBm(const Dev& dd, const TargetM<DIM>& tt, uint32_t tm, const double4& x, const double4& v,
                      const double4& e, float P, int type, const Inst* inst) : d(dd), t(tt), terms(tm), I(inst) {
        // the target's FP32 mirrors: the conversions of its v, rho, h and c
        const float4 vf = d.vf4[t.i], ef = d.ef4[t.i];
        vi[0] = vf.x; vi[1] = vf.y; vi[2] = vf.z;
        hi = ef.x; rhoi = vf.w; ci = ef.y; Pi = P; typei = type;
        solid_i = SOLID && is_solid_type(type);
        alpha = type > 100 ? d.av_alpha_solid_f : d.av_alpha_f;
        beta = type > 100 ? d.av_beta_solid_f : d.av_beta_f;
        psi = d.av_psi_f;
        skf = d.skf;
        kc = kconst_f_of<DIM>(d, t.i, skf, e.y);
        wd = 1.0f;
        Ri = make_float4(0, 0, 0, 0);
#pragma unroll
        for (int a = 0; a < DIM; ++a) aex[a] = 0.0;
        if ((terms & SPH_TERM_EXTERNAL) && (d.flags & SPH_F_GRAVITY) &&
            !((d.flags & SPH_F_GRAVITY_SKIP_SOLIDS) && type > 100))
            aex[DIM - 1] = d.gravity;
    }
    __device__ __forceinline__ void pair(int j) {
        const float4 pj = d.pr4[j];
        const float4 vj = d.vf4[j];
        const float4 ej = d.ef4[j];
        const float4 fj = d.pf4[j];
        float dx[3];
        rel_dx<DIM>(t, pj, dx);
        float dr = dx[0] * dx[0] + dx[1] * dx[1];
        if (DIM == 3) dr += dx[2] * dx[2];
        const float rinv = dr > 0.0f ? rsqrtf(dr) : 0.0f;
        const float q = (dr * rinv) * kc.hinv;
        const float g = kernel_g_f(skf, kc, q, rinv);
        const float mj = ej.w;
        const float vjv[3] = {vj.x, vj.y, vj.z};
        float w[DIM], dv[DIM];
        float dvw = 0.0f, xv = 0.0f;
#pragma unroll
        for (int a = 0; a < DIM; ++a) {
            w[a] = mj * (g * dx[a]);
            dv[a] = vi[a] - vjv[a];
            dvw = fmaf(dv[a], w[a], dvw);
            xv = fmaf(dx[a], dv[a], xv);
        }
        if (terms & SPH_TERM_INTERNAL) {
            const float aux = Pi + fj.x;
            float Tj[tf_stride_of(DIM)];
            load_tensor_f<DIM>((SOLID && solid_i) ? d.sf : d.tf, j, Tj);
#pragma unroll
            for (int a = 0; a < DIM; ++a) {
                float tsum = (SOLID && solid_i) ? 0.0f : -aux * w[a];
#pragma unroll
                for (int b = 0; b < DIM; ++b) tsum = fmaf(Tj[b * DIM + a], w[b], tsum);
                apsw[a].add(make_float2(tsum, w[a]));
            }
            ein.add(aux * dvw);
        }
        if ((terms & SPH_TERM_ARTI_VISC) && xv < 0.0f) {
            const float hij = 0.5f * (hi + ej.x);
            const float rij = 0.5f * (rhoi + vj.w);
            const float cij = 0.5f * (ci + ej.y);
            const float ph = psi * hij;
            const float phi = hij * xv / (dr + ph * ph);
            const float PI = (beta * phi - alpha * cij) * phi / rij;
            av01.add_prod(make_float2(-PI, -PI), make_float2(w[0], w[1]));
            if constexpr (DIM == 3) av2e.add_prod(make_float2(-PI, 0.5f * PI), make_float2(w[2], dvw));
            else av2e.add_prod(make_float2(0.5f * PI, 0.0f), make_float2(dvw, 0.0f));
        }
        if (terms & (SPH_TERM_EXTERNAL | SPH_TERM_ARTI_STRESS)) {
            const int tj = __float_as_int(fj.z);
            if ((terms & SPH_TERM_EXTERNAL) && typei > 0 && (tj < 0 || tj != typei) &&
                dr <= ext_reach2(*I, tj < 0, hi, ej.x))
                external_pair_f<DIM>(d, *I, dx, dr, hi, ci, typei, tj, ej.x, aexp);
            if (SOLID && DIM == 2 && (terms & SPH_TERM_ARTI_STRESS) && tj >= 100) {
                const float W = kernel_w_f(skf, kc, q);
                const float F = pow_int_or_real_f(W / wd, d.as_n_f);
                const float4 Rj = d.rf4[j];
                const float r00 = Ri.x + Rj.x, r11 = Ri.y + Rj.y, r01 = Ri.z + Rj.z;
                const float gx = g * dx[0], gy = g * dx[1];
                aas[0].add((mj * F) * (r00 * gx + r01 * gy));
                aas[DIM > 1 ? 1 : 0].add((mj * F) * (r01 * gx + r11 * gy));
            }
        }
    }
};

template <int DIM, bool SOLID, int K>
__device__ __forceinline__ void pass_b_mixed_targets(const Dev& d, int i, uint32_t terms, int assemble, uint32_t* lst,
                                                     float4* tile) {
    constexpr int D2 = DIM * DIM;
    const bool valid = i < d.n_real;
    const int ii = valid ? i : 0;
    const double4 xm = d.xm[ii];
    const double4 vr = d.vr[ii];
    const double4 eh = d.eh[ii];
    const int4 meta = d.meta[ii];
    const Target<DIM> tc = make_target<DIM>(d, ii, xm, eh.y);
    const TargetM<DIM> t = make_target_m<DIM>(d, ii, eh.y);
    PhysBm<DIM, SOLID> ph(d, t, terms, xm, vr, eh, d.pf4[ii].x, meta.x, &inst_of(d, ii));
    if (SOLID && DIM == 2 && (terms & SPH_TERM_ARTI_STRESS)) {
        ph.wd = kernel_w_f(d.skf, ph.kc, (float)(inst_of(d, ii).as_dp / eh.y));
        ph.Ri = d.rf4[ii];
    }
    walk_tiled<DIM, K>(d, tc, valid && meta.w != -1, ph, lst, tile, t.reach2);
    if (!valid) return;

    double a[DIM];
    double de = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) a[k] = 0.0;
    if (terms & SPH_TERM_INTERNAL) {
        const float* Ti = ((SOLID && ph.solid_i) ? d.sf : d.tf) + (size_t)i * tf_stride_of(DIM);
        float swv[DIM];
#pragma unroll
        for (int b = 0; b < DIM; ++b) swv[b] = ph.apsw[b].yf();
#pragma unroll
        for (int r = 0; r < DIM; ++r) {
            float s = 0.0f;
#pragma unroll
            for (int b = 0; b < DIM; ++b) s = fmaf(Ti[b * DIM + r], swv[b], s);
            a[r] = ph.apv(r) + (double)s;
        }
        de = d.tds[i] + 0.5 * ph.ein.value();
    }
    if (terms & SPH_TERM_ARTI_VISC) {
#pragma unroll
        for (int k = 0; k < DIM; ++k) a[k] += ph.aavv(k);
        de += ph.eavv();
    }
    if (terms & SPH_TERM_EXTERNAL) {
#pragma unroll
        for (int k = 0; k < DIM; ++k) a[k] += ph.aex[k] + ph.aexp[k].value();
    }
    if (terms & SPH_TERM_ARTI_STRESS) {
#pragma unroll
        for (int k = 0; k < DIM; ++k) a[k] += ph.aas[k].value();
    }
    if (assemble && meta.y == 1) {
#pragma unroll
        for (int k = 0; k < DIM; ++k) a[k] = 0.0;
    }
    double4 out = d.dvr[i];
    out.x = a[0];
    out.y = DIM > 1 ? a[1] : 0.0;
    out.z = DIM > 2 ? a[2] : 0.0;
    d.dvr[i] = out;
    d.dedt[i] = de;
}

template <int DIM, bool SOLID, int K, bool PERSIST>
__global__ void __launch_bounds__(MAX_TILE_TPB, DIM == 2 ? MIXED_B_MINB_2D : 4) pass_b_mixed_kernel(const Dev d, uint32_t terms, int assemble) {
    extern __shared__ uint32_t smem[];
    uint32_t* lst = smem + (threadIdx.x >> 5) * tiled_slot(K);
    float4* tile = reinterpret_cast<float4*>(lst + K * 32);
    if constexpr (PERSIST) {
        for (int base = blockIdx.x * blockDim.x; base < d.n_real; base += gridDim.x * blockDim.x)
            pass_b_mixed_targets<DIM, SOLID, K>(d, base + (int)threadIdx.x, terms, assemble, lst, tile);
    } else {
        pass_b_mixed_targets<DIM, SOLID, K>(d, (int)(blockIdx.x * blockDim.x + threadIdx.x), terms, assemble, lst, tile);
    }
}

// ---------------------------------------------------------------------------
// hash keys, reorder + half kick
// ---------------------------------------------------------------------------
// mark: bit 31 of a value flags a particle outside its grid (cell_of
// clamped it), for permute_kernel (indices stay below 2^31).
__global__ void keys_kernel(const Dev d, int n, const double4* __restrict__ xm, const int4* __restrict__ meta,
                            const int* __restrict__ pinst, uint32_t* __restrict__ keys,
                            uint32_t* __restrict__ vals, int* __restrict__ counts, int mark) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    double4 p = xm[s];
    double x[3] = {p.x, p.y, p.z};
    const Inst& I = d.inst[pinst[s]];
    int c[3];
    bool clamped;
    cell_of(I.grid, d.dim, x, c, &clamped);
    uint32_t key;
    if (!I.active) key = (uint32_t)d.total_cells + 1u;              // removed instance: dropped
    else if (meta[s].w == -1) key = (uint32_t)d.total_cells;        // State == -1: never a neighbour
    else {
        key = (uint32_t)(I.cell_base + cell_key(I.grid, c));
        atomicAdd(&counts[key], 1);
        if (clamped) atomicOr(d.status, ST_RANGE);
    }
    keys[s] = key;
    vals[s] = (uint32_t)s | (mark && clamped ? 0x80000000u : 0u);
}

__device__ __forceinline__ bool shear_type(int t) { return t >= 101 && t <= 104; }

// radial return (timeIntegration.f90:145-167)
template <int D2>
__device__ __forceinline__ void yield_scale(const DevMaterial* m, double* S) {
    if (!m || !m->yield) return;
    double J2 = 0.0;
#pragma unroll
    for (int k = 0; k < D2; ++k) J2 += S[k] * S[k];
    const double f = fmin(1.0, sqrt(((m->sigma_y * m->sigma_y) / 3) / J2));
#pragma unroll
    for (int k = 0; k < D2; ++k) S[k] *= f;
}

__device__ __forceinline__ float4 to_posf(const Grid& g, int dim, const double4& x) {
    double p[3] = {x.x, x.y, x.z};
    int c[3];
    bool clamped;
    cell_of(g, dim, p, c, &clamped);
    return make_float4((float)(x.x - g.lo[0]), (float)(x.y - g.lo[1]),
                       dim == 3 ? (float)(x.z - g.lo[2]) : 0.0f, clamped ? 1.0f : 0.0f);
}

// to_posf and write_mirrors of particle s from one cell_of, with the
// conversions to FP32 on the integer pipes (d2f): the values of those two,
// for permute_kernel, which the FP64 pipe binds (about 85 % busy; the
// conversion instructions and cell_of's compares issue there).
// The cell comes from the sorted key and the outside flag from bit 31 of the
// sorted value (keys_kernel's cell_of on the same position), so permute runs
// no cell_of of its own.
template <int DIM>
__device__ __forceinline__ void posf_and_mirrors(const Dev& d, const Grid& g, int base, int s, const double4& xm,
                                                 const double4& vr, const double4& eh, bool clamped) {
    const double x[3] = {xm.x, xm.y, xm.z};
    int c[3];
    cell_from_key(g, base, d.keys_s[s], c);
    d.posf[s] = make_float4(d2f(xm.x - g.lo[0]), d2f(xm.y - g.lo[1]), DIM == 3 ? d2f(xm.z - g.lo[2]) : 0.0f,
                            clamped ? 1.0f : 0.0f);
    if (d.precision == SPH_PREC_MIXED) {
        float r[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) r[a] = a < DIM ? d2f(x[a] - (g.lo[a] + (double)c[a] * g.cs)) : 0.0f;
        d.pr4[s] = make_float4(r[0], r[1], r[2], __int_as_float(cell_code(c)));
        d.vf4[s] = make_float4(d2f(vr.x), d2f(vr.y), d2f(vr.z), d2f(vr.w));
        d.ef4[s] = make_float4(d2f(eh.y), d2f(eh.z), d2f(eh.w), d2f(xm.w));
    } else if (d.precision == SPH_PREC_DF64) {
        write_df_mirrors(d, g, s, xm, vr, eh);
    }
}

template <int DIM, bool SOLID>
__global__ void permute_kernel(const Dev d, int kick) {
    const bool carry = !kick;
    constexpr int D2 = DIM * DIM;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.n_real) return;
    const uint32_t sv = d.vals_s[s];
    const int src = (int)(sv & 0x7fffffffu);   // bit 31: outside the grid (keys_kernel)
    double4 xm = d.xm[src];
    double4 vr = d.vr[src];
    double4 eh = d.eh[src];
    const int4 meta = d.meta[src];
    const int inst = d.pinst[src];
    const Inst& I = d.inst[inst];
    const double dt = I.dt;
    if (d.pold) d.pold[s] = d.pa4[src].y;
    kick = kick && I.step > 0;  // no half kick before an instance's first step
    const bool sumd = d.flags & SPH_F_SUM_DENSITY;
    double S[D2];
    if (SOLID) {
#pragma unroll
        for (int k = 0; k < D2; ++k) S[k] = d.shear[(size_t)src * D2 + k];
    }
    if (kick) {
        const double4 r = d.dvr[src];
        const double de = d.dedt[src];
        d.prev_e[s] = eh.x;
        eh.x = eh.x + (dt / 2) * de;
        if (eh.x < 0) eh.x = 0;
        double prho = vr.w;
        if (!sumd) vr.w = vr.w + (dt / 2) * r.w;
        d.prev_vr[s] = make_double4(vr.x, vr.y, vr.z, prho);
        vr.x = vr.x + (dt / 2) * r.x;
        vr.y = vr.y + (dt / 2) * r.y;
        if (DIM == 3) vr.z = vr.z + (dt / 2) * r.z;
        if (SOLID && shear_type(meta.x)) {
#pragma unroll
            for (int k = 0; k < D2; ++k) {
                d.shear_prev[(size_t)s * D2 + k] = S[k];
                S[k] = S[k] + (dt / 2) * d.dsdt[(size_t)src * D2 + k];
            }
            yield_scale<D2>(material_of(d, I, meta.x), S);
        }
    }
    eh.w = xm.w / vr.w;  // m / rho of the kicked state
    d.pinst2[s] = inst;
    if (carry) {  // no kick this reorder: the rates move with their particles
        d.dvr2[s] = d.dvr[src];
        d.dedt2[s] = d.dedt[src];
        if (SOLID) {
#pragma unroll
            for (int k = 0; k < D2; ++k) d.dsdt2[(size_t)s * D2 + k] = d.dsdt[(size_t)src * D2 + k];
        }
    }
    if (d.dxp) d.dxp2[s] = d.dxp[src];
    d.xm2[s] = xm;
    d.vr2[s] = vr;
    d.eh2[s] = eh;
    d.dsp2[s] = d.dsp[src];
    d.meta2[s] = meta;
    if (SOLID) {
#pragma unroll
        for (int k = 0; k < D2; ++k) d.shear2[(size_t)s * D2 + k] = S[k];
    }
    posf_and_mirrors<DIM>(d, I.grid, I.cell_base, s, xm, vr, eh, (sv >> 31) != 0u);
}

// ---------------------------------------------------------------------------
// leap-frog update + Courant reduction
// ---------------------------------------------------------------------------
template <int DIM, bool SOLID>
__global__ void __launch_bounds__(256, 4) update_kernel(const Dev d) {
    constexpr int D2 = DIM * DIM;
    __shared__ double smax[8], ssum[8];
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    double cn = 0.0;
    bool have = false;
    int inst = -1;
    if (s < d.n_real) {
        inst = d.pinst[s];
        const Inst& I = d.inst[inst];
        const double dt = I.dt;
        const bool first = I.step == 0;
        const bool sumd = d.flags & SPH_F_SUM_DENSITY;
        double4 xm = d.xm[s];
        double4 vr = d.vr[s];
        double4 eh = d.eh[s];
        double4 dp = d.dsp[s];
        const double4 r = d.dvr[s];
        const double de = d.dedt[s];
        const int type = d.meta[s].x;
        const bool xsph = d.flags & SPH_F_AVER_VELOCITY;
        if (d.sle) {
            // h_upgrade at the end of single_step (hsml.f90:8-38), on the
            // state the pair passes saw; the Courant number below uses it
            if (d.sle == 1) {
                eh.y = 2.0 * pow(xm.w / vr.w, 1.0 / DIM);
            } else {
                const double dh = (eh.y / DIM) * d.pa4[s].z;
                eh.y = eh.y + dt * dh;
                if (eh.y <= 0) eh.y = eh.y - dt * dh;
            }
            // the neighbours of the next search must stay within one cell
            if (eh.y * (double)d.scale_k > I.grid.cs) atomicOr(d.status, ST_H_RANGE);
        }
        const double4 av = xsph ? d.aver[s] : make_double4(0, 0, 0, 0);
        double v[3] = {vr.x, vr.y, vr.z};
        const double dv[3] = {r.x, r.y, r.z};
        const double avv[3] = {av.x, av.y, av.z};
        double x[3] = {xm.x, xm.y, xm.z};
        double ds[3] = {dp.x, dp.y, dp.z};
        if (first) {
            eh.x = eh.x + (dt / 2) * de;
            if (eh.x < 0) eh.x = 0;
            if (!sumd) vr.w = vr.w + (dt / 2) * r.w;
#pragma unroll
            for (int a = 0; a < DIM; ++a) {
                v[a] = xsph ? v[a] + (dt / 2) * dv[a] + avv[a] : v[a] + (dt / 2) * dv[a];
                ds[a] = dt * v[a];
                x[a] = x[a] + ds[a];
            }
        } else {
            const double4 pv = d.prev_vr[s];
            const double pvv[3] = {pv.x, pv.y, pv.z};
            eh.x = d.prev_e[s] + dt * de;
            if (eh.x < 0) eh.x = 0;
            if (!sumd) vr.w = pv.w + dt * r.w;
#pragma unroll
            for (int a = 0; a < DIM; ++a) {
                // (without XSPH the correction is +0.0: no add, no FP64 issue)
                v[a] = xsph ? pvv[a] + dt * dv[a] + avv[a] : pvv[a] + dt * dv[a];
                ds[a] = ds[a] + dt * v[a];
                x[a] = x[a] + dt * v[a];
            }
        }
        if (SOLID && shear_type(type)) {
            double S[D2];
#pragma unroll
            for (int k = 0; k < D2; ++k) {
                const double dsd = d.dsdt[(size_t)s * D2 + k];
                S[k] = first ? d.shear[(size_t)s * D2 + k] + (dt / 2) * dsd
                             : d.shear_prev[(size_t)s * D2 + k] + dt * dsd;
            }
            yield_scale<D2>(material_of(d, I, type), S);
#pragma unroll
            for (int k = 0; k < D2; ++k) d.shear[(size_t)s * D2 + k] = S[k];
        }
        vr.x = v[0]; vr.y = v[1]; vr.z = DIM == 3 ? v[2] : 0.0;
        xm.x = x[0]; xm.y = x[1]; if (DIM == 3) xm.z = x[2];
        dp.x = ds[0]; dp.y = ds[1]; if (DIM == 3) dp.z = ds[2];
        d.xm[s] = xm;
        d.vr[s] = vr;
        d.eh[s] = eh;
        d.dsp[s] = dp;
        bool fin = finite_d(vr.w) && finite_d(eh.x);
#pragma unroll
        for (int a = 0; a < DIM; ++a) fin = fin && finite_d(v[a]) && finite_d(x[a]);
        if (!fin) atomicOr(d.status, ST_NONFINITE);
        if (!first) {
            // courant_num (courantNumber.f90:27-29), 1.2 is a single literal
            const double divv = d.pa4[s].z;
            const double hs = eh.y, c = eh.z;
            cn = dt * (hs * divv + c + (double)1.2f * (d.cour_alpha * c + d.cour_beta * hs * fabs(divv))) / hs;
            have = true;
        }
    }
    // Courant max per instance by atomics (the max does not depend on their
    // order); the sum in a fixed order: a block that holds one instance (the
    // usual case) leaves its partial sum, a block that holds several leaves
    // its particles' numbers, and courant_final_kernel adds them up
    __shared__ int s_binst;
    if (threadIdx.x == 0) s_binst = inst;
    __syncthreads();
    const int binst = s_binst;
    const bool uniform = __syncthreads_and(inst < 0 || inst == binst);
    if (!uniform) {
        if (have) atomicMax(&d.cmax[inst], (unsigned long long)__double_as_longlong(cn));
        if (s < d.n_real) d.cnp[s] = have ? cn : 0.0;
        if (threadIdx.x == 0) d.cpinst[blockIdx.x] = -2;
        return;
    }
    // The max on the integer pipes (this kernel is bound by the FP64 pipe,
    // where fmax issues): non-negative doubles order like their bit patterns
    // and negative ones like negative integers, and the block's maximum starts
    // at 0, so a signed 64-bit max of the patterns (NaN taken as 0, which fmax
    // ignores) leaves the block the maximum fmax gives.
    long long mk = 0;
    if (have) {
        const long long b = __double_as_longlong(cn);
        mk = (b & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL ? 0 : b;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mk = max(mk, __shfl_xor_sync(SPH_FULL_MASK, mk, o));
    const double mx = mk > 0 ? __longlong_as_double(mk) : 0.0;
    double sm = have ? cn : 0.0;
    sm = warp_sum(sm);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) { smax[w] = mx; ssum[w] = sm; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { a = fmax(a, smax[q]); b += ssum[q]; }
        if (binst >= 0) atomicMax(&d.cmax[binst], (unsigned long long)__double_as_longlong(a));
        d.cpart[blockIdx.x] = b;
        d.cpinst[blockIdx.x] = binst;
    }
}

// One block per instance: the sum of its update blocks' partial sums (and of
// the numbers of its particles in blocks shared with other instances), each
// thread over a fixed stride of blocks, then a fixed tree; the instance's
// particles are the contiguous range of its cells [cell_base, +ncells).  Its
// first thread then closes the instance's step: the Courant statistics, the
// step counter and the time.
__global__ void __launch_bounds__(1024) courant_final_kernel(const Dev d) {
    constexpr int UB = 256;  // threads per update_kernel block
    __shared__ double red[1024];
    const int k = blockIdx.x;
    Inst& I = d.inst[k];
    double acc = 0.0;
    if (d.n_real > 0 && I.active && I.step > 0) {
        const int start = d.fstart[I.cell_base], end = d.fstart[I.cell_base + I.grid.ncells];
        if (end > start) {
            for (int b = start / UB + (int)threadIdx.x; b <= (end - 1) / UB; b += blockDim.x) {
                const int bi = d.cpinst[b];
                if (bi == k) {
                    acc += d.cpart[b];
                } else if (bi == -2) {
                    const int lo = max(b * UB, start), hi = min(b * UB + UB, end);
                    for (int s = lo; s < hi; ++s) acc += d.cnp[s];
                }
            }
        }
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x != 0 || !I.active) return;
    if (I.step > 0) {
        const double mx = __longlong_as_double((long long)d.cmax[k]);
        const double sm = red[0];
        d.cres[3 * k] = mx;
        // the mean is not reset between steps in the reference
        // (timeIntegration.f90:213-251)
        d.cres[3 * k + 1] = I.n_real > 0 ? (d.cres[3 * k + 1] + sm) / I.n_real : 0.0;
        d.cres[3 * k + 2] = sm;
    }
    d.cmax[k] = 0ull;
    I.step += 1;
    I.time += I.dt;
}

// ---------------------------------------------------------------------------
// neighbour counts / export (same walk and test as the passes)
// ---------------------------------------------------------------------------
struct CountPhys {
    int n = 0;
    __device__ __forceinline__ void pair(int) { ++n; }
};
struct ExportPhys {
    const Dev& d;
    int* out;
    int k = 0;
    __device__ ExportPhys(const Dev& dd, int* o) : d(dd), out(o) {}
    __device__ __forceinline__ void pair(int j) { out[k++] = d.meta[j].z + 1; }
};

template <int DIM>
__global__ void __launch_bounds__(TPB) count_kernel(const Dev d, int* counts) {
    constexpr int K = ListLen<DIM>::K;
    extern __shared__ uint32_t smem[];
    uint32_t* lst = smem + (threadIdx.x >> 5) * ListLen<DIM>::SLOT;
    float4* tile = reinterpret_cast<float4*>(lst + K * 32);
    const int i = blockIdx.x * TPB + threadIdx.x;
    const bool valid = i < d.n_real;
    const int ii = valid ? i : 0;
    const double4 xm = d.xm[ii];
    const double4 eh = d.eh[ii];
    const int4 meta = d.meta[ii];
    Target<DIM> t = make_target<DIM>(d, ii, xm, eh.y);
    CountPhys ph;
    walk_lane<DIM, K>(d, t, valid && meta.w != -1, ph, lst, ExactAccept<DIM>{d, t});
    if (valid) counts[meta.z] = ph.n;
}

template <int DIM>
__global__ void __launch_bounds__(TPB) export_kernel(const Dev d, const long long* offsets, int* list) {
    constexpr int K = ListLen<DIM>::K;
    extern __shared__ uint32_t smem[];
    uint32_t* lst = smem + (threadIdx.x >> 5) * ListLen<DIM>::SLOT;
    float4* tile = reinterpret_cast<float4*>(lst + K * 32);
    const int i = blockIdx.x * TPB + threadIdx.x;
    const bool valid = i < d.n_real;
    const int ii = valid ? i : 0;
    const double4 xm = d.xm[ii];
    const double4 eh = d.eh[ii];
    const int4 meta = d.meta[ii];
    Target<DIM> t = make_target<DIM>(d, ii, xm, eh.y);
    ExportPhys ph(d, list + (valid ? offsets[meta.z] : 0));
    walk_lane<DIM, K>(d, t, valid && meta.w != -1, ph, lst, ExactAccept<DIM>{d, t});
}

// ---------------------------------------------------------------------------
// upload / download
// ---------------------------------------------------------------------------
// Slot of the k-th particle of the combined range [0, n_real + n_wall):
// real particles first, then the wall region.
__device__ __forceinline__ int slot_of(const Dev& d, int k) {
    return k < d.n_real ? k : d.wall_off + (k - d.n_real);
}

// Device-side case generation: particle q of the concatenated blocks
// (real blocks first) into the staging columns of an upload:
// x[q*dim+a], v[q*dim+a], sc = [mass | rho | p | e | c | h] (N each),
// t3 = [type | state | boundary] (N each); wall order = identity.
__global__ void generate_blocks_kernel(const sph_block* __restrict__ blocks, const int64_t* __restrict__ start,
                                       int nb, int dim, int64_t N, int64_t n_r, double* __restrict__ x,
                                       double* __restrict__ v, double* __restrict__ sc, int* __restrict__ t3,
                                       uint32_t* __restrict__ wall_order) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= N) return;
    int b = 0;
    while (b + 1 < nb && start[b + 1] <= q) ++b;
    const sph_block& B = blocks[b];
    const int64_t l = q - start[b];
    const int64_t n1 = dim > 1 ? B.n[1] : 1, n2 = dim > 2 ? B.n[2] : 1;
    const int64_t idx[3] = {l / (n1 * n2), (l / n2) % n1, l % n2};
    double xq[3] = {0.0, 0.0, 0.0};
    for (int a = 0; a < dim; ++a)  // origin + (i + 1/2) spacing, rounded as written
        xq[a] = __dadd_rn(B.origin[a], __dmul_rn((double)idx[a] + 0.5, B.spacing[a]));
    double p = 0.0;
    if (B.p_rho0_g != 0.0) p = __dmul_rn(B.p_rho0_g, fmax(__dsub_rn(B.p_level, xq[B.up_axis]), 0.0));
    const double rho = B.tait_b > 0.0
        ? pow(__dadd_rn(__ddiv_rn(p, B.tait_b), 1.0), 1.0 / B.tait_gamma) * B.tait_rho0
        : B.rho;
    const double xc = xq[B.clamp_axis];
    const bool clamped = xc < B.clamp_below || xc > B.clamp_above;
    for (int a = 0; a < dim; ++a) {
        double va = B.v[a];
        if (B.v_ramp_len > 0.0) va = va + __ddiv_rn(__dmul_rn(B.v_ramp[a], fmax(xq[0], 0.0)), B.v_ramp_len);
        x[q * dim + a] = xq[a];
        v[q * dim + a] = clamped ? 0.0 : va;
    }
    sc[q] = B.mass;
    sc[N + q] = rho;
    sc[2 * N + q] = p;
    sc[3 * N + q] = 0.0;
    sc[4 * N + q] = B.c;
    sc[5 * N + q] = B.h;
    t3[q] = B.type;
    t3[N + q] = B.state;
    t3[2 * N + q] = clamped ? 1 : 0;
    if (q >= n_r) wall_order[q - n_r] = (uint32_t)(q - n_r);
}

// One instance's upload: its n_r real particles go to slots [real_dst, +n_r)
// in the uploaded order, its n_w walls to [wall_dst, +n_w) in their cell
// order (wall_order).  meta.z keeps the index within the upload.
__global__ void pack_kernel(const Dev d, int n_r, int n_w, int real_dst, int wall_dst, int inst_id,
                            const double* __restrict__ x, const double* __restrict__ v,
                            const double* __restrict__ m, const double* __restrict__ rho,
                            const double* __restrict__ p, const double* __restrict__ e,
                            const double* __restrict__ c, const double* __restrict__ h,
                            const int* __restrict__ type, const int* __restrict__ state,
                            const int* __restrict__ bnd, const double* __restrict__ shear,
                            const uint32_t* __restrict__ wall_order) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_r + n_w) return;
    const int src = k < n_r ? k : n_r + (int)wall_order[k - n_r];
    const int s = k < n_r ? real_dst + k : wall_dst + (k - n_r);
    const int dim = d.dim, D2 = d.d2;
    const Grid& g = d.inst[inst_id].grid;
    double4 xm = make_double4(x[(size_t)src * dim], dim > 1 ? x[(size_t)src * dim + 1] : 0.0,
                              dim > 2 ? x[(size_t)src * dim + 2] : 0.0, m[src]);
    double4 vr = make_double4(v[(size_t)src * dim], dim > 1 ? v[(size_t)src * dim + 1] : 0.0,
                              dim > 2 ? v[(size_t)src * dim + 2] : 0.0, rho[src]);
    double4 eh = make_double4(e[src], h[src], c[src], m[src] / rho[src]);
    int4 meta = make_int4(type[src], bnd ? bnd[src] : 0, src, state ? state[src] : 0);
    d.xm[s] = xm; d.vr[s] = vr; d.eh[s] = eh; d.meta[s] = meta;
    d.xm2[s] = xm; d.vr2[s] = vr; d.eh2[s] = eh; d.meta2[s] = meta;
    d.pinst[s] = inst_id; d.pinst2[s] = inst_id;
    d.dsp[s] = make_double4(0, 0, 0, 0);
    d.dsp2[s] = make_double4(0, 0, 0, 0);
    d.dvr[s] = make_double4(0, 0, 0, 0);
    d.dedt[s] = 0.0;
    if (d.dxp) { d.dxp[s] = 0.0; d.dxp2[s] = 0.0; }  // divergencePosition starts at 0
    if (d.aver) d.aver[s] = make_double4(0, 0, 0, 0);
    d.pa4[s] = make_double4(0.0, p[src], 0.0, 0.0);
    d.posf[s] = to_posf(g, dim, xm);
    write_mirrors(d, g, s, xm, vr, eh);
    if (d.precision == SPH_PREC_MIXED) {
        for (int q = 0; q < D2; ++q) d.tf[(size_t)s * d.tfs + q] = 0.0f;
        d.pf4[s] = make_float4(0.0f, (float)p[src], __int_as_float(meta.x), 0.0f);
    } else if (d.precision == SPH_PREC_DF64) {
        for (int q = 0; q < D2; ++q) d.ttd[(size_t)s * D2 + q] = make_float2(0.0f, 0.0f);
        float4 e1 = d.ed1[s];
        e1.z = e1.w = 0.0f;
        d.ed1[s] = e1;
    }
    for (int q = 0; q < D2; ++q) d.tt[(size_t)s * D2 + q] = 0.0;
    if (d.has_solid) {
        for (int q = 0; q < D2; ++q) {
            double sv = shear ? shear[(size_t)src * D2 + q] : 0.0;
            d.shear[(size_t)s * D2 + q] = sv;
            d.shear2[(size_t)s * D2 + q] = sv;
            d.sig[(size_t)s * D2 + q] = 0.0;
            d.dsdt[(size_t)s * D2 + q] = 0.0;
        }
        if (d.dim == 2) d.ras[s] = make_double4(0, 0, 0, 0);
    }
}

// Walls: EOS once (internal_force re-evaluates it every step on constant
// wall densities, internalForce.f90:103-134), p/rho^2 and stress/rho^2.
__global__ void wall_init_kernel(const Dev d, int first, int count) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= count) return;
    const int s = first + w;
    const int4 meta = d.meta[s];
    const Inst& I = inst_of(d, s);
    const double4 vr = d.vr[s];
    double4 eh = d.eh[s];
    double p = d.pa4[s].y, c = eh.z;
    if (d.wraw) d.wraw[s] = make_double2(p, c);
    const DevMaterial* m = material_of(d, I, meta.x);
    const bool solid = is_solid_type(meta.x);
    if (solid) solid_eos(m, vr.w, eh.x, p);
    else fluid_eos(m, vr.w, eh.x, p, c);
    const double rho2 = vr.w * vr.w;
    d.pa4[s] = make_double4(p / rho2, p, 0.0, 0.0);
    eh.z = c;
    d.eh[s] = eh;
    d.eh2[s] = eh;
    // a wall's tt: no viscous part, its pressure on the diagonal (SPH = 2)
    const double pd = d.pa_sph == 2 ? -(p / rho2) : 0.0;
    for (int k = 0; k < d.d2; ++k) d.tt[(size_t)s * d.d2 + k] = (k % (d.dim + 1) == 0) ? pd : 0.0;
    if (d.precision == SPH_PREC_DF64) {
        write_mirrors(d, I.grid, s, d.xm[s], vr, eh);
        const DF P = df_from(p / rho2), cc = df_from(c), PD = df_from(pd);
        d.ed1[s] = make_float4(cc.hi, cc.lo, P.hi, P.lo);
        for (int k = 0; k < d.d2; ++k)
            d.ttd[(size_t)s * d.d2 + k] = (k % (d.dim + 1) == 0) ? make_float2(PD.hi, PD.lo) : make_float2(0.0f, 0.0f);
    }
    if (d.precision == SPH_PREC_MIXED) {
        write_mirrors(d, I.grid, s, d.xm[s], vr, eh);
        d.pf4[s] = make_float4((float)(p / rho2), (float)p, __int_as_float(meta.x), 0.0f);
        for (int k = 0; k < d.d2; ++k) d.tf[(size_t)s * d.tfs + k] = 0.0f;
        if (d.has_solid) {
            for (int k = 0; k < d.d2; ++k) d.sf[(size_t)s * d.tfs + k] = 0.0f;
            if (solid)
                for (int a = 0; a < d.dim; ++a) d.sf[(size_t)s * d.tfs + a * d.dim + a] = (float)(-p / rho2);
        }
    }
    if (d.has_solid) {
        const int D2 = d.d2;
        for (int k = 0; k < D2; ++k) d.sig[(size_t)s * D2 + k] = 0.0;
        if (solid)
            for (int a = 0; a < d.dim; ++a) d.sig[(size_t)s * D2 + a * d.dim + a] = -p / rho2;
    }
}

__global__ void gather_kernel(const Dev d, int field, double* __restrict__ out, int inst_filter) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= d.n_real + d.n_wall) return;
    const int s = slot_of(d, k);
    if (inst_filter >= 0 && !slot_in_inst(d, s, inst_filter)) return;
    const int dim = d.dim, D2 = d.d2;
    const int4 meta = d.meta[s];
    const int o = meta.z;
    const bool real = s < d.n_real;
    switch (field) {
    case SPH_FIELD_X: { double4 v = d.xm[s]; for (int a = 0; a < dim; ++a) out[(size_t)o * dim + a] = cmp(v, a); } break;
    case SPH_FIELD_V: { double4 v = d.vr[s]; for (int a = 0; a < dim; ++a) out[(size_t)o * dim + a] = cmp(v, a); } break;
    case SPH_FIELD_MASS: out[o] = d.xm[s].w; break;
    case SPH_FIELD_RHO: out[o] = d.vr[s].w; break;
    case SPH_FIELD_P: out[o] = d.pa4[s].y; break;
    case SPH_FIELD_E: out[o] = d.eh[s].x; break;
    case SPH_FIELD_C: out[o] = d.eh[s].z; break;
    case SPH_FIELD_H: out[o] = d.eh[s].y; break;
    case SPH_FIELD_DIVX: out[o] = real ? d.pa4[s].w : 0.0; break;
    case SPH_FIELD_DIVV: out[o] = real ? d.pa4[s].z : 0.0; break;
    case SPH_FIELD_DISP: { double4 v = d.dsp[s]; for (int a = 0; a < dim; ++a) out[(size_t)o * dim + a] = real ? cmp(v, a) : 0.0; } break;
    case SPH_FIELD_DVDT: { double4 v = d.dvr[s]; for (int a = 0; a < dim; ++a) out[(size_t)o * dim + a] = real ? cmp(v, a) : 0.0; } break;
    case SPH_FIELD_DRHODT: out[o] = real ? d.dvr[s].w : 0.0; break;
    case SPH_FIELD_DEDT: out[o] = real ? d.dedt[s] : 0.0; break;
    case SPH_FIELD_NNEIGH: out[o] = real ? (double)d.nneigh[s] : 0.0; break;
    case SPH_FIELD_TYPE: out[o] = (double)meta.x; break;
    case SPH_FIELD_AVER: {
        const double4 v = (real && d.aver) ? d.aver[s] : make_double4(0, 0, 0, 0);
        for (int a = 0; a < dim; ++a) out[(size_t)o * dim + a] = cmp(v, a);
    } break;
    case SPH_FIELD_VISC: {
        const DevMaterial* m = material_of(d, inst_of(d, s), meta.x);
        out[o] = ((d.flags & SPH_F_VISCOSITY) && m) ? m->eta : 0.0;
    } break;
    case SPH_FIELD_SHEAR:
    case SPH_FIELD_DSDT:
    case SPH_FIELD_STRESS:
    case SPH_FIELD_STRAIN:
        for (int k = 0; k < D2; ++k) {
            double v = 0.0;
            if (field == SPH_FIELD_STRAIN) v = real ? d.strain[(size_t)s * D2 + k] : 0.0;
            else if (d.has_solid) {
                if (field == SPH_FIELD_SHEAR) v = d.shear[(size_t)s * D2 + k];
                else if (field == SPH_FIELD_DSDT) v = real ? d.dsdt[(size_t)s * D2 + k] : 0.0;
                else if (is_solid_type(meta.x)) {
                    v = d.shear[(size_t)s * D2 + k];
                    if (k % (dim + 1) == 0) v -= d.pa4[s].y;
                }
            }
            out[(size_t)o * D2 + k] = v;
        }
        break;
    default: break;
    }
}

__global__ void set_field_kernel(const Dev d, int field, const double* __restrict__ in, int limit,
                                 int inst_filter) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= d.n_real + d.n_wall) return;
    const int s = slot_of(d, k);
    if (inst_filter >= 0 && !slot_in_inst(d, s, inst_filter)) return;
    const int dim = d.dim, D2 = d.d2;
    const int o = d.meta[s].z;
    if (o >= limit) return;
    const Grid& g = inst_of(d, s).grid;
    const bool real = s < d.n_real;
    switch (field) {
    case SPH_FIELD_X: { double4 v = d.xm[s]; for (int a = 0; a < dim; ++a) setc(v, a, in[(size_t)o * dim + a]); d.xm[s] = v; d.posf[s] = to_posf(g, dim, v); } break;
    case SPH_FIELD_V: { double4 v = d.vr[s]; for (int a = 0; a < dim; ++a) setc(v, a, in[(size_t)o * dim + a]); d.vr[s] = v; } break;
    case SPH_FIELD_MASS: { double4 v = d.xm[s]; v.w = in[o]; d.xm[s] = v; double4 e = d.eh[s]; e.w = v.w / d.vr[s].w; d.eh[s] = e; } break;
    case SPH_FIELD_RHO: { double4 v = d.vr[s]; v.w = in[o]; d.vr[s] = v; double4 e = d.eh[s]; e.w = d.xm[s].w / v.w; d.eh[s] = e; } break;
    case SPH_FIELD_P: { double4 v = d.pa4[s]; v.y = in[o]; d.pa4[s] = v; } break;
    case SPH_FIELD_E: { double4 v = d.eh[s]; v.x = in[o]; d.eh[s] = v; } break;
    case SPH_FIELD_C: { double4 v = d.eh[s]; v.z = in[o]; d.eh[s] = v; } break;
    case SPH_FIELD_H: { double4 v = d.eh[s]; v.y = in[o]; d.eh[s] = v; } break;
    case SPH_FIELD_DIVX: if (real) { double4 v = d.pa4[s]; v.w = in[o]; d.pa4[s] = v; } break;
    case SPH_FIELD_DVDT: if (real) { double4 v = d.dvr[s]; for (int a = 0; a < dim; ++a) setc(v, a, in[(size_t)o * dim + a]); d.dvr[s] = v; } break;
    case SPH_FIELD_DRHODT: if (real) { double4 v = d.dvr[s]; v.w = in[o]; d.dvr[s] = v; } break;
    case SPH_FIELD_DEDT: if (real) d.dedt[s] = in[o]; break;
    case SPH_FIELD_SHEAR: if (d.has_solid) for (int k = 0; k < D2; ++k) d.shear[(size_t)s * D2 + k] = in[(size_t)o * D2 + k]; break;
    case SPH_FIELD_DSDT: if (d.has_solid && real) for (int k = 0; k < D2; ++k) d.dsdt[(size_t)s * D2 + k] = in[(size_t)o * D2 + k]; break;
    default: break;
    }
    write_mirrors(d, g, s, d.xm[s], d.vr[s], d.eh[s]);
}

// Real particles' (x, v, rho, e) between the uploaded order in `stage`
// ([x n*dim | v n*dim | rho n | e n]) and the cell order on the device.
// The reference constants (KRef) of instance `inst` for the h of its real
// particle `first` (none: first < 0), by the expressions the passes use.
template <int DIM>
__global__ void kref_kernel(const Dev d, int inst, int first) {
    KRef r{};
    r.skf = d.skf;
    if (first >= 0) {
        r.h = d.eh[first].y;
        r.k = make_kconst<DIM>(d.skf, r.h);
        r.kf = make_kconst_f<DIM>(d.skf, r.h);
        reach_bounds(d, d.inst[inst].grid, r.h, &r.reach, &r.lo2, &r.hi2);
        const float reach = (float)(r.h * (double)d.scale_k);
        r.reach2f = reach * reach;
    }
    const_cast<KRef*>(d.kref)[inst] = r;
}

// mode 0: state -> stage (upload order); 1: stage -> state; 2: the positions
// alone (what the cell keys read); 3: v, rho and e, after 2.  2 and 3 serve a
// call that steps at once: its reorder recomputes what depends on them (the
// FP32 positions, m / rho and the FP32 mirrors), so they write the uploaded
// values alone and leave that FP64 work (and the FP64 pipe) to the reorder.
__global__ void host_state_kernel(const Dev d, int mode, double* __restrict__ stage) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.n_real) return;
    const int dim = d.dim, nr = d.n_real;
    const int o = d.meta[s].z;
    double* X = stage;
    double* V = stage + (size_t)nr * dim;
    double* R = V + (size_t)nr * dim;
    double* E = R + nr;
    double4 xm = d.xm[s];
    if (mode == 2) {
        for (int a = 0; a < dim; ++a) setc(xm, a, X[(size_t)o * dim + a]);
        d.xm[s] = xm;
        return;
    }
    double4 vr = d.vr[s], eh = d.eh[s];
    if (mode == 3) {
        for (int a = 0; a < dim; ++a) setc(vr, a, V[(size_t)o * dim + a]);
        vr.w = R[o];
        eh.x = E[o];
        d.vr[s] = vr;
        d.eh[s] = eh;
        return;
    }
    if (mode == 1) {
        for (int a = 0; a < dim; ++a) {
            setc(xm, a, X[(size_t)o * dim + a]);
            setc(vr, a, V[(size_t)o * dim + a]);
        }
        vr.w = R[o];
        eh.x = E[o];
        eh.w = xm.w / vr.w;
        const Grid& g = inst_of(d, s).grid;
        d.xm[s] = xm;
        d.posf[s] = to_posf(g, d.dim, xm);
        d.vr[s] = vr; d.eh[s] = eh;
        write_mirrors(d, g, s, xm, vr, eh);
    } else {
        for (int a = 0; a < dim; ++a) { X[(size_t)o * dim + a] = cmp(xm, a); V[(size_t)o * dim + a] = cmp(vr, a); }
        R[o] = vr.w;
        E[o] = eh.x;
    }
}

// Energy sums over the real particles (of system `inst`, or all when inst <
// 0), in FP64: kinetic 1/2 m v.v, internal m e and, with gravity on,
// gravitational -m g x_(dim-1).  Each block leaves its three partial sums
// (warp shuffle tree, then its warps in order); energy_final_kernel adds the
// partials in a fixed order, so a state gives the same bits on every call.
constexpr int ENERGY_TPB = 256;
__global__ void __launch_bounds__(ENERGY_TPB) energy_partial_kernel(const Dev d, int inst, double* __restrict__ part) {
    __shared__ double ws[3][ENERGY_TPB / 32];
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    double k = 0.0, u = 0.0, g = 0.0;
    if (s < d.n_real && (inst < 0 || d.pinst[s] == inst)) {
        const double4 xm = d.xm[s], vr = d.vr[s];
        const double m = xm.w;
        double vv = vr.x * vr.x + vr.y * vr.y;
        if (d.dim == 3) vv += vr.z * vr.z;
        k = 0.5 * m * vv;
        u = m * d.eh[s].x;
        if (d.flags & SPH_F_GRAVITY) g = -(m * d.gravity) * (d.dim == 3 ? xm.z : xm.y);
    }
    k = warp_sum(k);
    u = warp_sum(u);
    g = warp_sum(g);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) { ws[0][w] = k; ws[1][w] = u; ws[2][w] = g; }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int q = 0; q < ENERGY_TPB / 32; ++q) t += ws[threadIdx.x][q];
        part[(size_t)blockIdx.x * 3 + threadIdx.x] = t;
    }
}

__global__ void __launch_bounds__(ENERGY_TPB) energy_final_kernel(const double* __restrict__ part, int nb,
                                                                   double* __restrict__ out) {
    __shared__ double ws[3][ENERGY_TPB / 32];
    double t[3] = {0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < nb; b += ENERGY_TPB)
        for (int c = 0; c < 3; ++c) t[c] += part[(size_t)b * 3 + c];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int c = 0; c < 3; ++c) {
        t[c] = warp_sum(t[c]);
        if (lane == 0) ws[c][w] = t[c];
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double v = 0.0;
        for (int q = 0; q < ENERGY_TPB / 32; ++q) v += ws[threadIdx.x][q];
        out[threadIdx.x] = v;
    }
}

// fixedBoundary (boundaryCondition.f90:32-45): the velocity rate of a
// particle with Boundary == 1 becomes zero, in a host-order array and in the
// assembled rates
__global__ void boundary_kernel(const Dev d, double* __restrict__ dv) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= d.n_real || d.meta[s].y != 1) return;
    if (dv)
        for (int a = 0; a < d.dim; ++a) dv[(size_t)d.meta[s].z * d.dim + a] = 0.0;
    double4 r = d.dvr[s];
    r.x = r.y = r.z = 0.0;
    d.dvr[s] = r;
}

// courant_num (courantNumber.f90:7-31), the expression of update_kernel
__global__ void courant_num_kernel(int n, double dt, double ca, double cb, const double* __restrict__ h,
                                   const double* __restrict__ dv, const double* __restrict__ c,
                                   double* __restrict__ xi) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double hs = h[i], divv = dv[i], ci = c[i];
    xi[i] = dt * (hs * divv + ci + (double)1.2f * (ca * ci + cb * hs * fabs(divv))) / hs;
}

__global__ void add_offset_kernel(int* a, int n, int off) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] += off;
}

// Dependent FP64 FMA chains held in registers: the FP64 issue-rate probe.
// d2f and f2d against the conversion instructions: case k of a seeded
// stream (splitmix64) in each class, mismatches counted.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
__global__ void conversion_check_kernel(int64_t n, uint64_t seed, unsigned long long* bad) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const unsigned long long r = mix64(seed ^ mix64((unsigned long long)k));
    const unsigned long long r2 = mix64(r);
    unsigned long long cases[5];
    cases[0] = r;                                                        // any bit pattern
    const unsigned long long e = 897ull + (r2 % 253ull);                 // float-normal exponents
    const unsigned long long inrange = (r & 0x800fffffffffffffull) | (e << 52);
    cases[1] = inrange;
    cases[2] = (inrange & ~0x1fffffffull) | 0x10000000ull;               // exactly half: ties
    cases[3] = (inrange & ~0x1fffffffull) | (0x10000000ull + ((r2 >> 40) & 1 ? 1ull : 0ull) - ((r2 >> 41) & 1 ? 1ull : 0ull));
    cases[4] = (r2 & 0x8000000000000000ull) | ((unsigned long long)(896 + 254) << 52) | (r & 0xfffffffffffffull);  // near FLT_MAX
    unsigned n_bad = 0;
    for (int c = 0; c < 5; ++c) {
        const double x = __longlong_as_double((long long)cases[c]);
        const float a = d2f(x), b = __double2float_rn(x);
        const bool same = __float_as_uint(a) == __float_as_uint(b) || (a != a && b != b);
        n_bad += same ? 0u : 1u;
    }
    const float f = __uint_as_float((uint32_t)r2);
    const double fa = f2d(f), fb = (double)f;
    n_bad += (__double_as_longlong(fa) == __double_as_longlong(fb) || (fa != fa && fb != fb)) ? 0u : 1u;
    if (n_bad) atomicAdd(bad, (unsigned long long)n_bad);
}

__global__ void fp64_probe_kernel(double* sink, int iters) {
    double a0 = threadIdx.x * 1e-9, a1 = a0 + 1e-9, a2 = a0 + 2e-9, a3 = a0 + 3e-9;
    double a4 = a0 + 4e-9, a5 = a0 + 5e-9, a6 = a0 + 6e-9, a7 = a0 + 7e-9;
    const double b = 0.9999999, c = 1e-9;
    for (int k = 0; k < iters; ++k) {
        a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
        a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
    }
    double s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
    if (s == 123.456) sink[0] = s;  // never true; keeps the chains live
}

inline unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

template <int DIM, bool TILED = false, bool SPLIT = false>
size_t list_smem() { return (size_t)WARPS * ListLen<DIM, TILED, SPLIT>::SLOT * sizeof(uint32_t); }

size_t tiled_smem(const Dev& d) { return (size_t)(d.tile_tpb / 32) * tiled_slot(d.tile_k) * sizeof(uint32_t); }

// The list lengths the tiled kernels are compiled for (SPH_OPT_LIST_LEN).
template <int V> using TileK = std::integral_constant<int, V>;
template <class F>
void with_tile_k(const Dev& d, F&& f) {
    switch (d.tile_k) {
    case 64: f(TileK<64>{}); break;
    case 120: f(TileK<120>{}); break;
    default: f(TileK<88>{}); break;
    }
}

}  // namespace

// Blocks of a launch of a tiled (mixed) pass: one per tile of d.tile_tpb
// targets, or, for a persistent launch (d.persistent), as many as the device
// holds at once, each striding over the tiles.
template <class Kern>
static unsigned tiled_grid(const Dev& d, Kern kern) {
    const unsigned tiles = nblk(d.n_real, d.tile_tpb);
    if (!d.persistent) return tiles;
    int dev = 0, sms = 0, per = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, d.tile_tpb, tiled_smem(d)) != cudaSuccess ||
        per < 1) {
        cudaGetLastError();
        return tiles;
    }
    return std::min<unsigned>(tiles, (unsigned)per * (unsigned)sms);
}

uint32_t step_terms(const Dev& d) {
    uint32_t t = SPH_TERM_INTERNAL;
    if (d.flags & SPH_F_ARTI_VISC) t |= SPH_TERM_ARTI_VISC;
    if (d.flags & (SPH_F_EXT_FORCE | SPH_F_DUMMY | SPH_F_GRAVITY)) t |= SPH_TERM_EXTERNAL;
    if ((d.flags & SPH_F_ARTI_STRESS) && d.dim == 2) t |= SPH_TERM_ARTI_STRESS;
    if (d.flags & SPH_F_ARTI_HEAT) t |= SPH_TERM_ARTI_HEAT;
    return t;
}

void launch_keys(const Dev& d, int n, const double4* xm, const int4* meta, const int* pinst, uint32_t* keys,
                 uint32_t* vals, int* counts, cudaStream_t s, bool mark_outside) {
    if (n <= 0) return;
    keys_kernel<<<nblk(n, 256), 256, 0, s>>>(d, n, xm, meta, pinst, keys, vals, counts, mark_outside ? 1 : 0);
}

void launch_permute(const Dev& d, bool kick, cudaStream_t s) {
    if (d.n_real <= 0) return;
    const unsigned g = nblk(d.n_real, 256);
    if (d.dim == 2) {
        if (d.has_solid) permute_kernel<2, true><<<g, 256, 0, s>>>(d, kick);
        else permute_kernel<2, false><<<g, 256, 0, s>>>(d, kick);
    } else {
        if (d.has_solid) permute_kernel<3, true><<<g, 256, 0, s>>>(d, kick);
        else permute_kernel<3, false><<<g, 256, 0, s>>>(d, kick);
    }
}

void launch_kernel_correction(const Dev& d, cudaStream_t s) {
    if (d.n_real <= 0 || !d.kgc) return;
    if (d.dim == 2) pass_k_kernel<2><<<nblk(d.n_real, TPB), TPB, list_smem<2>(), s>>>(d);
    else pass_k_kernel<3><<<nblk(d.n_real, TPB), TPB, list_smem<3>(), s>>>(d);
}

void launch_density(const Dev& d, cudaStream_t s) {
    if (d.n_real <= 0) return;
    const unsigned g = nblk(d.n_real, TPB);
    if (d.dim == 2) {
        if (d.precision == SPH_PREC_MIXED) with_tile_k(d, [&](auto k) {
            if (d.persistent) {
                auto kern = pass_s_mixed_kernel<2, decltype(k)::value, true>;
                kern<<<tiled_grid(d, kern), d.tile_tpb, tiled_smem(d), s>>>(d);
            } else {
                pass_s_mixed_kernel<2, decltype(k)::value, false><<<nblk(d.n_real, d.tile_tpb), d.tile_tpb, tiled_smem(d), s>>>(d);
            }
        });
        else pass_s_kernel<2><<<g, TPB, list_smem<2>(), s>>>(d);
    } else {
        if (d.precision == SPH_PREC_MIXED) with_tile_k(d, [&](auto k) {
            if (d.persistent) {
                auto kern = pass_s_mixed_kernel<3, decltype(k)::value, true>;
                kern<<<tiled_grid(d, kern), d.tile_tpb, tiled_smem(d), s>>>(d);
            } else {
                pass_s_mixed_kernel<3, decltype(k)::value, false><<<nblk(d.n_real, d.tile_tpb), d.tile_tpb, tiled_smem(d), s>>>(d);
            }
        });
        else pass_s_kernel<3><<<g, TPB, list_smem<3>(), s>>>(d);
    }
    density_apply_kernel<<<nblk(d.n_real, 256), 256, 0, s>>>(d);
}

// SPH_OPT_LANES applies to the FP64 passes A and B of the SPH = 2 form
// without kernel correction or artificial heat, while the lanes of all
// targets fit a 32-bit thread index; the other forms run one lane per target.
static bool lanes_apply(const Dev& d) {
    return d.lane_shift > 0 && d.precision == SPH_PREC_FP64 && !d.kgc && d.pa_sph == 2 &&
           !(d.flags & SPH_F_ARTI_HEAT) && ((long long)d.n_real << d.lane_shift) <= 0x7fffffffLL;
}

template <int DIM, bool SOLID>
static void pass_a_t(const Dev& d, bool want_strain, cudaStream_t s) {
    // XSPH is a template flag: its sums stay out of the registers of the
    // walk when the option is off
    const bool xs = d.flags & SPH_F_AVER_VELOCITY;
    auto go = [&](auto kern) {
        kern<<<nblk(d.n_real, TPB), TPB, list_smem<DIM, true>(), s>>>(d, want_strain ? 1 : 0);
    };
    if (lanes_apply(d)) {
        auto kern = xs ? pass_a_kernel<DIM, SOLID, false, false, true, true>
                       : pass_a_kernel<DIM, SOLID, false, false, false, true>;
        kern<<<nblk((long long)d.n_real << d.lane_shift, TPB), TPB, list_smem<DIM, true>(), s>>>(d, want_strain ? 1 : 0);
    } else if (!SOLID && d.precision == SPH_PREC_DF64) {
        if (xs) go(pass_a_kernel<DIM, false, false, true, true>);
        else go(pass_a_kernel<DIM, false, false, true>);
    } else if (SOLID && d.kgc) {
        if (xs) go(pass_a_kernel<DIM, SOLID, true, false, true>);
        else go(pass_a_kernel<DIM, SOLID, true>);
    } else if (d.precision == SPH_PREC_MIXED) {
        with_tile_k(d, [&](auto k) {
            if (d.persistent) {
                auto kern = pass_a_mixed_kernel<DIM, SOLID, decltype(k)::value, true>;
                kern<<<tiled_grid(d, kern), d.tile_tpb, tiled_smem(d), s>>>(d, want_strain ? 1 : 0);
            } else {
                pass_a_mixed_kernel<DIM, SOLID, decltype(k)::value, false>
                    <<<nblk(d.n_real, d.tile_tpb), d.tile_tpb, tiled_smem(d), s>>>(d, want_strain ? 1 : 0);
            }
        });
    } else if (xs) {
        go(pass_a_kernel<DIM, SOLID, false, false, true>);
    } else {
        go(pass_a_kernel<DIM, SOLID>);
    }
}

void launch_riemann_density(const Dev& d, cudaStream_t s) {
    if (d.n_real <= 0) return;
    if (d.dim == 2) pass_r_kernel<2><<<nblk(d.n_real, TPB), TPB, list_smem<2>(), s>>>(d);
    else pass_r_kernel<3><<<nblk(d.n_real, TPB), TPB, list_smem<3>(), s>>>(d);
}

void launch_pass_a(const Dev& d, bool want_strain, cudaStream_t s) {
    if (d.n_real <= 0) return;
    if (d.dim == 2) { if (d.has_solid) pass_a_t<2, true>(d, want_strain, s); else pass_a_t<2, false>(d, want_strain, s); }
    else { if (d.has_solid) pass_a_t<3, true>(d, want_strain, s); else pass_a_t<3, false>(d, want_strain, s); }
}

template <int DIM, bool SOLID>
static void pass_b_t(const Dev& d, uint32_t terms, bool assemble, cudaStream_t s) {
    if (lanes_apply(d))
        pass_b_kernel<DIM, SOLID, false, false, 2, false, true>
            <<<nblk((long long)d.n_real << d.lane_shift, TPB), TPB, list_smem<DIM, true, true>(), s>>>(d, terms, assemble ? 1 : 0);
    else if (!SOLID && d.precision == SPH_PREC_DF64)
        pass_b_kernel<DIM, false, false, true><<<nblk(d.n_real, TPB), TPB, list_smem<DIM, true, true>(), s>>>(d, terms, assemble ? 1 : 0);
    else if (SOLID && d.kgc)
        pass_b_kernel<DIM, SOLID, true><<<nblk(d.n_real, TPB), TPB, list_smem<DIM, true, true>(), s>>>(d, terms, assemble ? 1 : 0);
    else if (d.pa_sph == 1)
        pass_b_kernel<DIM, SOLID, false, false, 1><<<nblk(d.n_real, TPB), TPB, list_smem<DIM, true, true>(), s>>>(d, terms, assemble ? 1 : 0);
    else if (d.pa_sph == 3)
        pass_b_kernel<DIM, SOLID, false, false, 3><<<nblk(d.n_real, TPB), TPB, list_smem<DIM, true, true>(), s>>>(d, terms, assemble ? 1 : 0);
    else if (terms & SPH_TERM_ARTI_HEAT)   // FP64, SPH = 2, no correction (sph_params check)
        pass_b_kernel<DIM, SOLID, false, false, 2, true><<<nblk(d.n_real, TPB), TPB, list_smem<DIM, true, true>(), s>>>(d, terms, assemble ? 1 : 0);
    else if (d.precision == SPH_PREC_MIXED)
        with_tile_k(d, [&](auto k) {
            if (d.persistent) {
                auto kern = pass_b_mixed_kernel<DIM, SOLID, decltype(k)::value, true>;
                kern<<<tiled_grid(d, kern), d.tile_tpb, tiled_smem(d), s>>>(d, terms, assemble ? 1 : 0);
            } else {
                pass_b_mixed_kernel<DIM, SOLID, decltype(k)::value, false>
                    <<<nblk(d.n_real, d.tile_tpb), d.tile_tpb, tiled_smem(d), s>>>(d, terms, assemble ? 1 : 0);
            }
        });
    else
        pass_b_kernel<DIM, SOLID><<<nblk(d.n_real, TPB), TPB, list_smem<DIM, true, true>(), s>>>(d, terms, assemble ? 1 : 0);
}

void launch_pass_b(const Dev& d, uint32_t terms, bool assemble, cudaStream_t s) {
    if (d.n_real <= 0) return;
    if (d.dim == 2) { if (d.has_solid) pass_b_t<2, true>(d, terms, assemble, s); else pass_b_t<2, false>(d, terms, assemble, s); }
    else { if (d.has_solid) pass_b_t<3, true>(d, terms, assemble, s); else pass_b_t<3, false>(d, terms, assemble, s); }
}

void launch_update(const Dev& d, cudaStream_t s) {
    if (d.n_real > 0) {
        const unsigned g = nblk(d.n_real, 256);
        if (d.dim == 2) {
            if (d.has_solid) update_kernel<2, true><<<g, 256, 0, s>>>(d);
            else update_kernel<2, false><<<g, 256, 0, s>>>(d);
        } else {
            if (d.has_solid) update_kernel<3, true><<<g, 256, 0, s>>>(d);
            else update_kernel<3, false><<<g, 256, 0, s>>>(d);
        }
    }
    if (d.n_inst > 0) courant_final_kernel<<<d.n_inst, 1024, 0, s>>>(d);
}

void launch_count_neighbors(const Dev& d, int* counts, cudaStream_t s) {
    if (d.n_real <= 0) return;
    if (d.dim == 2) count_kernel<2><<<nblk(d.n_real, TPB), TPB, list_smem<2>(), s>>>(d, counts);
    else count_kernel<3><<<nblk(d.n_real, TPB), TPB, list_smem<3>(), s>>>(d, counts);
}

void launch_export_neighbors(const Dev& d, const long long* offsets, int* list, cudaStream_t s) {
    if (d.n_real <= 0) return;
    if (d.dim == 2) export_kernel<2><<<nblk(d.n_real, TPB), TPB, list_smem<2>(), s>>>(d, offsets, list);
    else export_kernel<3><<<nblk(d.n_real, TPB), TPB, list_smem<3>(), s>>>(d, offsets, list);
}

void launch_wall_init(const Dev& d, int first, int count, cudaStream_t s) {
    if (count <= 0) return;
    wall_init_kernel<<<nblk(count, 256), 256, 0, s>>>(d, first, count);
}

void launch_pack_upload(const Dev& d, int n_r, int n_w, int real_dst, int wall_dst, int inst_id,
                        const double* x, const double* v, const double* m, const double* rho, const double* p,
                        const double* e, const double* c, const double* h, const int* type, const int* state,
                        const int* bnd, const double* shear, const uint32_t* wall_order, cudaStream_t s) {
    if (n_r + n_w <= 0) return;
    pack_kernel<<<nblk(n_r + n_w, 256), 256, 0, s>>>(d, n_r, n_w, real_dst, wall_dst, inst_id, x, v, m, rho, p,
                                                      e, c, h, type, state, bnd, shear, wall_order);
}

void launch_gather_field(const Dev& d, int field, double* out, int inst_filter, cudaStream_t s) {
    if (d.n_real + d.n_wall <= 0) return;
    gather_kernel<<<nblk(d.n_real + d.n_wall, 256), 256, 0, s>>>(d, field, out, inst_filter);
}

void launch_set_field(const Dev& d, int field, const double* in, int limit, int inst_filter, cudaStream_t s) {
    if (d.n_real + d.n_wall <= 0) return;
    set_field_kernel<<<nblk(d.n_real + d.n_wall, 256), 256, 0, s>>>(d, field, in, limit, inst_filter);
}

void launch_boundary(const Dev& d, double* dv, cudaStream_t s) {
    if (d.n_real <= 0) return;
    boundary_kernel<<<nblk(d.n_real, 256), 256, 0, s>>>(d, dv);
}

void launch_courant_num(int n, double dt, double ca, double cb, const double* h, const double* dv,
                        const double* c, double* xi, cudaStream_t s) {
    if (n <= 0) return;
    courant_num_kernel<<<nblk(n, 256), 256, 0, s>>>(n, dt, ca, cb, h, dv, c, xi);
}

int launch_energy(const Dev& d, int inst, double* part, double* out, cudaStream_t s) {
    const int nb = d.n_real > 0 ? (int)nblk(d.n_real, ENERGY_TPB) : 0;
    if (nb > 0) energy_partial_kernel<<<nb, ENERGY_TPB, 0, s>>>(d, inst, part);
    energy_final_kernel<<<1, ENERGY_TPB, 0, s>>>(part, nb, out);
    return nb > 0 ? 2 : 1;
}

void launch_kref(const Dev& d, int inst, int first, cudaStream_t s) {
    if (d.dim == 2) kref_kernel<2><<<1, 1, 0, s>>>(d, inst, first);
    else kref_kernel<3><<<1, 1, 0, s>>>(d, inst, first);
}

void launch_host_state(const Dev& d, int mode, double* stage, cudaStream_t s) {
    if (d.n_real <= 0) return;
    host_state_kernel<<<nblk(d.n_real, 256), 256, 0, s>>>(d, mode, stage);
}

template <int DIM, bool SOLID, bool P>
static void set_mixed_carveout_t(int v) {
    cudaFuncSetAttribute(pass_a_mixed_kernel<DIM, SOLID, 64, P>, cudaFuncAttributePreferredSharedMemoryCarveout, v);
    cudaFuncSetAttribute(pass_b_mixed_kernel<DIM, SOLID, 64, P>, cudaFuncAttributePreferredSharedMemoryCarveout, v);
    cudaFuncSetAttribute(pass_a_mixed_kernel<DIM, SOLID, 88, P>, cudaFuncAttributePreferredSharedMemoryCarveout, v);
    cudaFuncSetAttribute(pass_b_mixed_kernel<DIM, SOLID, 88, P>, cudaFuncAttributePreferredSharedMemoryCarveout, v);
    cudaFuncSetAttribute(pass_a_mixed_kernel<DIM, SOLID, 120, P>, cudaFuncAttributePreferredSharedMemoryCarveout, v);
    cudaFuncSetAttribute(pass_b_mixed_kernel<DIM, SOLID, 120, P>, cudaFuncAttributePreferredSharedMemoryCarveout, v);
}

template <int DIM, bool SOLID>
static void set_carveout_t(int v) {
    cudaFuncSetAttribute(pass_a_kernel<DIM, SOLID>, cudaFuncAttributePreferredSharedMemoryCarveout, v);
    cudaFuncSetAttribute(pass_a_kernel<DIM, SOLID, false, false, true>, cudaFuncAttributePreferredSharedMemoryCarveout, v);
    cudaFuncSetAttribute(pass_b_kernel<DIM, SOLID>, cudaFuncAttributePreferredSharedMemoryCarveout, v);
    cudaFuncSetAttribute(pass_a_kernel<DIM, SOLID, false, false, false, true>, cudaFuncAttributePreferredSharedMemoryCarveout, v);
    cudaFuncSetAttribute(pass_a_kernel<DIM, SOLID, false, false, true, true>, cudaFuncAttributePreferredSharedMemoryCarveout, v);
    cudaFuncSetAttribute(pass_b_kernel<DIM, SOLID, false, false, 2, false, true>, cudaFuncAttributePreferredSharedMemoryCarveout, v);
    set_mixed_carveout_t<DIM, SOLID, false>(v);
    set_mixed_carveout_t<DIM, SOLID, true>(v);
}

void set_pass_carveout(int percent) {
    const int v = percent < 0 ? (int)cudaSharedmemCarveoutDefault : (percent > 100 ? 100 : percent);
    set_carveout_t<2, false>(v);
    set_carveout_t<2, true>(v);
    set_carveout_t<3, false>(v);
    set_carveout_t<3, true>(v);
    cudaGetLastError();
}

template <int DIM, bool SOLID, int K>
static void set_tiled_smem_t(int bytes) {
    cudaFuncSetAttribute(pass_a_mixed_kernel<DIM, SOLID, K, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(pass_b_mixed_kernel<DIM, SOLID, K, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(pass_a_mixed_kernel<DIM, SOLID, K, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(pass_b_mixed_kernel<DIM, SOLID, K, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (!SOLID) {
        cudaFuncSetAttribute(pass_s_mixed_kernel<DIM, K, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        cudaFuncSetAttribute(pass_s_mixed_kernel<DIM, K, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    }
}

template <int K>
static void set_tiled_smem_k(int bytes) {
    set_tiled_smem_t<2, false, K>(bytes);
    set_tiled_smem_t<2, true, K>(bytes);
    set_tiled_smem_t<3, false, K>(bytes);
    set_tiled_smem_t<3, true, K>(bytes);
}

int set_tiled_smem_limit(size_t bytes) {
    const int b = (int)bytes;
    set_tiled_smem_k<64>(b);
    set_tiled_smem_k<88>(b);
    set_tiled_smem_k<120>(b);
    return (int)cudaGetLastError();
}

size_t tiled_smem_bytes(int tpb, int k) { return (size_t)(tpb / 32) * tiled_slot(k) * sizeof(uint32_t); }

int default_tile_k(int dim) { return dim == 2 ? ListLen<2, true>::K : ListLen<3, true>::K; }

void launch_generate_blocks(const sph_block* blocks, const int64_t* start, int nb, int dim, int64_t N,
                            int64_t n_r, double* x, double* v, double* sc, int* t3, uint32_t* wall_order,
                            cudaStream_t s) {
    if (N <= 0) return;
    generate_blocks_kernel<<<nblk(N, 256), 256, 0, s>>>(blocks, start, nb, dim, N, n_r, x, v, sc, t3, wall_order);
}

void launch_add_offset(int* a, int64_t n, int off, cudaStream_t s) {
    if (n <= 0 || off == 0) return;
    add_offset_kernel<<<nblk(n, 256), 256, 0, s>>>(a, (int)n, off);
}

void launch_conversion_check(int64_t n, uint64_t seed, unsigned long long* bad, cudaStream_t s) {
    if (n > 0) conversion_check_kernel<<<nblk(n, 256), 256, 0, s>>>(n, seed, bad);
}

void launch_fp64_probe(double* sink, int iters, int blocks, cudaStream_t s) {
    fp64_probe_kernel<<<blocks, 256, 0, s>>>(sink, iters);
}

}  // namespace sph
