// strip.cu -- warp-strip step kernels of the synthetic-workload (CFG) physics.
//
// Each warp owns a 128-cell-wide strip of R consecutive rows of one group: a
// lane holds four consecutive cells and moves them with 128-bit loads and
// stores; the rows above and below roll through registers, east and west
// neighbours come from warp shuffles (plus one scalar load at each end of the
// strip).  Per cell-update the forward step then touches u(k) once, u(k-1) once,
// the coefficient once and writes u(k+1) once -- the 16 bytes the update needs
// -- with a handful of instructions.  The adjoint step rolls z(k+1), the
// coefficient and the forward slice u(q) the same way and keeps the
// correlation update to one 128-bit read-modify-write per four cells.
//
// The forward launch also carries the sensor gather of slice k in one extra
// block per group (it reads slice k, which is complete), replacing a separate
// launch per step.  Same arithmetic, operand order and results as the per-cell
// kernels in kernels.cu.
#include <cuda_runtime.h>

#include <cstdint>

#include "internal.h"

namespace tomo {
namespace {

#include "cell.cuh"

constexpr int STRIP = 128;     // cells per warp strip
constexpr int WARPS = 4;       // warps per block (stacked in y)

// West neighbour of element 0 and east neighbour of element 3 of each lane.
__device__ __forceinline__ void we(const float4& v, const float* __restrict__ row, int lane, int x0, int nx,
                                   float& west, float& east) {
    west = __shfl_up_sync(FULL, v.w, 1);
    east = __shfl_down_sync(FULL, v.x, 1);
    if (lane == 0) west = x0 > 0 ? row[x0 - 1] : 0.f;
    if (lane == 31) east = x0 + STRIP < nx ? row[x0 + STRIP] : 0.f;
}

// ---------------------------------------------------------------------------
template <int R>
__global__ void __launch_bounds__(WARPS * 32) k_fwd_strip(DevGeo g, const float* __restrict__ coef, FwdStep s) {
    const int nx = g.nx, ny = g.ny;
    const int gl = blockIdx.z;
    if (blockIdx.y == gridDim.y - 1) {
        // sensor gather of slice k (k >= 2), one block per group
        if (blockIdx.x != 0 || s.gk < 2) return;
        const float* u = s.uc + gl * s.gstride;
        const int64_t base = ((int64_t)gl * g.nt + s.gk) * g.nch;
        const bool noisy = s.gmeas && g.noise_key;
        const uint64_t key = noisy ? *g.noise_key : 0;
        for (int c = threadIdx.x; c < g.nch; c += blockDim.x) {
            const int cell = g.rcv[c];
            float v = cell >= 0 ? u[cell] : 0.f;
            if (noisy) v *= noise_factor(key, g.noise_level, s.g0 + gl, s.gk, c);
            s.gout[base + c] = s.gmeas ? (cell >= 0 ? s.gmeas[base + c] - v : 0.f) : v;
        }
        return;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x0 = blockIdx.x * STRIP;
    const int i = x0 + 4 * lane;
    const int y0 = (blockIdx.y * WARPS + warp) * R;
    if (y0 >= ny) return;
    const bool act = i < nx;
    const float* uc = s.uc + gl * s.gstride;
    const float* up = s.up + gl * s.gstride;
    float* un = s.un + gl * s.gstride;
    float* ck = s.ck ? s.ck + gl * s.ckstride : nullptr;
    const bool edge_x = x0 < g.sponge_w || x0 + STRIP > nx - g.sponge_w;
    const bool src = s.k < g.n_src_steps;
    const int32_t* em = g.emit + (int64_t)(s.g0 + gl) * g.gs;
    const float a = src ? g.src[s.k] : 0.f;
    float4 rm = ld4(uc, (int64_t)(y0 - 1) * nx + i, act && y0 > 0);
    float4 r0 = ld4(uc, (int64_t)y0 * nx + i, act);
#pragma unroll 4
    for (int r = 0; r < R; ++r) {
        const int j = y0 + r;
        if (j >= ny) break;
        const int64_t row = (int64_t)j * nx;
        const float4 rp = ld4(uc, row + nx + i, act && j + 1 < ny);
        const float4 p = ld4(up, row + i, act);
        const float4 c = ld4(coef, row + i, act);
        float w, e;
        we(r0, uc + row, lane, x0, nx, w, e);
        const bool near = edge_x || j < g.sponge_w || j >= ny - g.sponge_w;
        const float dx = near ? sponge(g, i, j) : 1.f;
        const float dy = near ? sponge(g, i + 1, j) : 1.f;
        const float dz = near ? sponge(g, i + 2, j) : 1.f;
        const float dw = near ? sponge(g, i + 3, j) : 1.f;
        const int64_t q0 = row + i;
        const float ax = src ? emit_at(em, g.gs, q0, a) : 0.f;
        const float ay = src ? emit_at(em, g.gs, q0 + 1, a) : 0.f;
        const float az = src ? emit_at(em, g.gs, q0 + 2, a) : 0.f;
        const float aw = src ? emit_at(em, g.gs, q0 + 3, a) : 0.f;
        float4 v;
        v.x = fwd_cell(r0.y, w, rm.x, rp.x, r0.x, p.x, c.x, dx, ax);
        v.y = fwd_cell(r0.z, r0.x, rm.y, rp.y, r0.y, p.y, c.y, dy, ay);
        v.z = fwd_cell(r0.w, r0.y, rm.z, rp.z, r0.z, p.z, c.z, dz, az);
        v.w = fwd_cell(e, r0.z, rm.w, rp.w, r0.w, p.w, c.w, dw, aw);
        if (act) {
            *reinterpret_cast<float4*>(un + row + i) = v;
            if (ck) *reinterpret_cast<float4*>(ck + row + i) = v;
        }
        rm = r0;
        r0 = rp;
    }
}

// ---------------------------------------------------------------------------
// MINB: minimum resident blocks per SM requested from the register allocator
// (8 caps registers at 64 per thread); UNR: unroll factor of the row loop.
template <int R, int MINB, int UNR>
__global__ void __launch_bounds__(WARPS * 32, MINB) k_adj_strip(DevGeo g, const float* __restrict__ coef,
                                                               AdjStep s) {
    const int nx = g.nx, ny = g.ny;
    const int gl = blockIdx.z;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x0 = blockIdx.x * STRIP;
    const int i = x0 + 4 * lane;
    const int y0 = (blockIdx.y * WARPS + warp) * R;
    if (y0 >= ny) return;
    const bool act = i < nx;
    const float* z1 = s.z1 + gl * s.zstride;
    const float* z2 = s.z2 + gl * s.zstride;
    float* zk = s.zk + gl * s.zstride;
    const float* u = s.uq + gl * s.ustride;
    const float* rr = s.rr + gl * s.rrstride;
    float* corr = s.corr + gl * s.cstride;
    const bool edge_x = x0 < g.sponge_w || x0 + STRIP > nx - g.sponge_w;
    const RcvMask rk = rcv_mask(g, x0, x0 + STRIP);
    const int dc[4] = {edge_dist(i, nx), edge_dist(i + 1, nx), edge_dist(i + 2, nx), edge_dist(i + 3, nx)};
    // rolling rows: the products c*z(k+1) above and at the row, z(k+1) and u at the row, u above
    // (32-bit offsets: the strip path requires nx*ny < 2^31)
    const bool up_ok = act && y0 > 0;
    const int top = (y0 - 1) * nx + i;
    float4 pm = mul4(ld4(coef, top, up_ok), ld4(z1, top, up_ok));
    float4 z0 = ld4(z1, y0 * nx + i, act);
    float4 p0 = mul4(ld4(coef, y0 * nx + i, act), z0);
    float4 um = ld4(u, top, up_ok);
    float4 u0 = ld4(u, y0 * nx + i, act);
#pragma unroll UNR
    for (int r = 0; r < R; ++r) {
        const int j = y0 + r;
        if (j >= ny) break;
        const int row = j * nx;
        const bool has_next = act && j + 1 < ny;
        const float4 zp = ld4(z1, row + nx + i, has_next);
        const float4 pp = mul4(ld4(coef, row + nx + i, has_next), zp);
        const float4 uq = ld4(u, row + nx + i, has_next);
        const float4 zz = ld4(z2, row + i, act);
        // products at the west/east neighbours via shuffles, one scalar pair at each strip end
        float pw = __shfl_up_sync(FULL, p0.w, 1), pe = __shfl_down_sync(FULL, p0.x, 1);
        if (lane == 0) pw = x0 > 0 ? mul(coef[row + x0 - 1], z1[row + x0 - 1]) : 0.f;
        if (lane == 31) pe = x0 + STRIP < nx ? mul(coef[row + x0 + STRIP], z1[row + x0 + STRIP]) : 0.f;
        const float ps[4] = {pm.x, pm.y, pm.z, pm.w};
        const float pn[4] = {pp.x, pp.y, pp.z, pp.w};
        const float pe4[4] = {p0.y, p0.z, p0.w, pe};
        const float pw4[4] = {pw, p0.x, p0.y, p0.z};
        const float pc[4] = {p0.x, p0.y, p0.z, p0.w};
        const float zc[4] = {z0.x, z0.y, z0.z, z0.w};
        const float z2v[4] = {zz.x, zz.y, zz.z, zz.w};
        const bool near_y = j < g.sponge_w || j >= ny - g.sponge_w;
        const int dr = edge_dist(j, ny);
        int4 rid = make_int4(-1, -1, -1, -1);
        if (rcv_row(g, rk, j) && act) rid = *reinterpret_cast<const int4*>(g.rid + row + i);
        const int rids[4] = {rid.x, rid.y, rid.z, rid.w};
        float v[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const float inj = rids[t] >= 0 ? rr[rids[t]] : 0.f;
            float d = 1.f;
            if (edge_x || near_y) d = damp_at(g, dc[t], dr);
            v[t] = adj_cell(pe4[t], pw4[t], ps[t], pn[t], pc[t], zc[t], z2v[t], inj, d);
        }
        // Laplacian of the forward slice (zero outside the grid)
        float uw, ue;
        we(u0, u + row, lane, x0, nx, uw, ue);
        const float uus[4] = {um.x, um.y, um.z, um.w};
        const float uun[4] = {uq.x, uq.y, uq.z, uq.w};
        const float uc4[4] = {u0.x, u0.y, u0.z, u0.w};
        const float uue[4] = {u0.y, u0.z, u0.w, ue};
        const float uuw[4] = {uw, u0.x, u0.y, u0.z};
        if (act) {
            float4 cr = *reinterpret_cast<const float4*>(corr + row + i);
            float lu[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) lu[t] = lap5(uue[t], uuw[t], uus[t], uun[t], uc4[t]);
            cr.x = __fmaf_rn(v[0], lu[0], cr.x);
            cr.y = __fmaf_rn(v[1], lu[1], cr.y);
            cr.z = __fmaf_rn(v[2], lu[2], cr.z);
            cr.w = __fmaf_rn(v[3], lu[3], cr.w);
            *reinterpret_cast<float4*>(corr + row + i) = cr;
            *reinterpret_cast<float4*>(zk + row + i) = make_float4(v[0], v[1], v[2], v[3]);
        }
        pm = p0; p0 = pp; z0 = zp;
        um = u0; u0 = uq;
    }
}

// part[(g0+gl)*nt + k] = sum_c rr(gl, k, c)^2, one block per (k, group), fixed order.
__global__ void __launch_bounds__(256) k_resid_parts(const float* __restrict__ rr, int nt, int nch, double* part) {
    const int k = blockIdx.x, gl = blockIdx.y;
    const float* r = rr + ((int64_t)gl * nt + k) * nch;
    double acc = 0.0;
    for (int c = threadIdx.x; c < nch; c += 256) acc += (double)r[c] * (double)r[c];
    __shared__ double red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[(int64_t)gl * nt + k] = red[0];
}

// ---------------------------------------------------------------------------
// Two adjoint steps per launch (temporal blocking in registers).  A lane holds
// two cells; strips are 64 cells wide and overlap by one lane (2 cells) on each
// side, so lanes 0 and 31 compute the first step as halo for their neighbours
// and only lanes 1..30 (60 cells) write.  Rows y0-1 .. y0+R of the first step
// z(kz) roll through registers and the second step z(kz-1) is computed one row
// behind.  Both slices, and the correlation with u(q) and u(q-1), are written
// once per launch: per cell-update this moves z(kz+1), z(kz+2), u(q), u(q-1),
// the coefficient and the correlation once per two steps.  The z ring has four
// slots, so the second step never overwrites a slice another warp still reads.
// Both kernels evaluate cells with adj_cell/lap5 and fused correlation updates,
// so the results are identical to two one-step launches.
struct Adj2Step {
    const float* z2;    // z(kz+2)
    const float* z1;    // z(kz+1)
    float* za;          // z(kz)   out
    float* zb;          // z(kz-1) out
    int64_t zstride;
    const float* ua;    // u(q)   correlated with z(kz)
    const float* ub;    // u(q-1) correlated with z(kz-1)
    int64_t ustride;
    const float* rra;   // residual of pass-group 0 at step kz
    const float* rrb;   // at step kz-1
    int64_t rrstride;
    float* corr;
    int64_t cstride;
    int ng;
};

__device__ __forceinline__ float2 ld2(const float* __restrict__ p, int64_t off, bool ok) {
    return ok ? *reinterpret_cast<const float2*>(p + off) : make_float2(0.f, 0.f);
}

// Rows y0 .. y0+R-1 of one warp strip.  EDGE = false: the strip, its one-cell halo and rows
// y0-2 .. y0+R+2 lie inside the grid, so no access needs a bounds predicate.
template <int R, int AHEAD, bool EDGE, bool PACK>
__device__ __forceinline__ void adj2_rows(const DevGeo& g, const float* __restrict__ coef, const Adj2Step& s,
                                          int x0, int y0) {
    constexpr bool PF = AHEAD >= 1;
    const int nx = g.nx, ny = g.ny;
    const int gl = blockIdx.z;
    const int lane = threadIdx.x & 31;
    const int i = x0 + 2 * lane;
    const bool in = !EDGE || (i >= 0 && i < nx);
    const bool own = in && lane >= 1 && lane <= 30;
    const int yend = min(y0 + R, ny);          // rows y0 .. yend-1 are written
    const float* z1 = s.z1 + gl * s.zstride;
    const float* z2 = s.z2 + gl * s.zstride;
    float* za = s.za + gl * s.zstride;
    float* zb = s.zb + gl * s.zstride;
    const float* ua = s.ua + gl * s.ustride;
    const float* ub = s.ub + gl * s.ustride;
    const float* rra = s.rra + gl * s.rrstride;
    const float* rrb = s.rrb + gl * s.rrstride;
    float* corr = s.corr + gl * s.cstride;
    const bool edge_x = x0 < g.sponge_w || x0 + 64 > nx - g.sponge_w;
    auto row_ok = [&](int r) { return !EDGE || (in && r >= 0 && r < ny); };
    const RcvMask rk = rcv_mask(g, x0, x0 + 64);
    const int dca = edge_dist(i, nx), dcb = edge_dist(i + 1, nx);
    // rolling state at the top of iteration r (first step at row r, second at row r-1), with
    // 32-bit offsets (the strip path requires nx*ny < 2^31):
    //   z(kz+1) at rows r-1 (z1m) and r (z10); products c*z(kz+1) at rows r-1, r (pzm, pz0);
    //   the coefficient at row r (c0); z(kz) at row r-1 (zam) and its products c*z(kz) at
    //   rows r-2, r-1 (pam2, pam); u(q), u(q-1) at rows r-2, r-1; receiver ids of row r-1;
    //   the correlation of row r-1 (read one iteration ahead)
    float2 z1m = ld2(z1, (y0 - 2) * nx + i, row_ok(y0 - 2));
    float2 z10 = ld2(z1, (y0 - 1) * nx + i, row_ok(y0 - 1));
    float2 pzm = mul2(ld2(coef, (y0 - 2) * nx + i, row_ok(y0 - 2)), z1m);
    float2 c0 = ld2(coef, (y0 - 1) * nx + i, row_ok(y0 - 1));
    float2 pz0 = mul2(c0, z10);
    float2 zam = make_float2(0.f, 0.f), pam2 = make_float2(0.f, 0.f), pam = make_float2(0.f, 0.f);
    float2 uam2 = make_float2(0.f, 0.f), uam = make_float2(0.f, 0.f);
    float2 ubm2 = make_float2(0.f, 0.f), ubm = make_float2(0.f, 0.f);
    float2 crm = make_float2(0.f, 0.f);
    int2 ridm = make_int2(-1, -1);
    bool rcvm = false;                         // row r-1 has receivers in the strip
    // AHEAD == 2: the inputs of the coming iteration (rows r+1 of z(kz+1) and the coefficient,
    // rows r of z(kz+2), u(q), u(q-1) and the receiver ids)
    float2 q_z1 = make_float2(0.f, 0.f), q_c = q_z1, q_zz = q_z1, q_ua = q_z1, q_ub = q_z1;
    int2 q_rid = make_int2(-1, -1);
    bool q_rcv = false;
    if (AHEAD == 2) {
        const int r = y0 - 1, row = r * nx;
        q_z1 = ld2(z1, row + nx + i, row_ok(r + 1));
        q_c = ld2(coef, row + nx + i, row_ok(r + 1));
        q_zz = ld2(z2, row + i, row_ok(r));
        q_ua = ld2(ua, row + i, row_ok(r));
        q_ub = ld2(ub, row + i, row_ok(r));
        q_rcv = rcv_row(g, rk, r);
        if (q_rcv && row_ok(r)) q_rid = *reinterpret_cast<const int2*>(g.rid + row + i);
    }
#pragma unroll 1
    for (int r = y0 - 1; r <= y0 + R; ++r) {
        if (EDGE && r > ny) break;
        const int row = r * nx;
        const bool ok = row_ok(r);
        float2 z1p, cp, zz, ua0, ub0;
        int2 rid = make_int2(-1, -1);
        bool rcv;
        if (AHEAD == 2) {
            z1p = q_z1; cp = q_c; zz = q_zz; ua0 = q_ua; ub0 = q_ub; rid = q_rid; rcv = q_rcv;
            const int rn = r + 1, rown = row + nx;
            q_z1 = ld2(z1, rown + nx + i, row_ok(rn + 1));
            q_c = ld2(coef, rown + nx + i, row_ok(rn + 1));
            q_zz = ld2(z2, rown + i, row_ok(rn));
            q_ua = ld2(ua, rown + i, row_ok(rn));
            q_ub = ld2(ub, rown + i, row_ok(rn));
            q_rid = make_int2(-1, -1);
            q_rcv = rcv_row(g, rk, rn);
            if (q_rcv && row_ok(rn)) q_rid = *reinterpret_cast<const int2*>(g.rid + rown + i);
        } else {
            const bool okn = row_ok(r + 1);
            z1p = ld2(z1, row + nx + i, okn);
            cp = ld2(coef, row + nx + i, okn);
            zz = ld2(z2, row + i, ok);
            ua0 = ld2(ua, row + i, ok);
            ub0 = ld2(ub, row + i, ok);
            rcv = rcv_row(g, rk, r);
            if (rcv && ok) rid = *reinterpret_cast<const int2*>(g.rid + row + i);
        }
        // correlation of row r, read now for the second step of the next iteration
        float2 cr_next = make_float2(0.f, 0.f);
        if (PF && own && r >= y0 && r < yend) cr_next = *reinterpret_cast<const float2*>(corr + row + i);
        const float2 pzp = PACK ? pk_mul(cp, z1p) : mul2(cp, z1p);
        // ---- first step: z(kz) at row r (all lanes; zero outside the grid)
        float2 za0 = make_float2(0.f, 0.f);
        {
            // lane 0's west and lane 31's east neighbour come from no lane: only the halo cells
            // x0 and x0+63, whose first-step values no owned cell reads, would use them
            const float pw = __shfl_up_sync(FULL, pz0.y, 1), pe = __shfl_down_sync(FULL, pz0.x, 1);
            if (ok) {
                const int dr = edge_dist(r, ny);
                const float drow = dr < g.sponge_w ? g.damp[dr] : 1.f;
                float dx = drow, dy = drow;
                if (edge_x) { dx = damp_at(g, dca, dr); dy = damp_at(g, dcb, dr); }
                float ix = 0.f, iy = 0.f;
                if (rcv) {
                    ix = rid.x >= 0 ? rra[rid.x] : 0.f;
                    iy = rid.y >= 0 ? rra[rid.y] : 0.f;
                }
                if constexpr (PACK) {
                    za0 = adj_cell2(make_float2(pz0.y, pe), make_float2(pw, pz0.x), pzm, pzp, pz0, z10, zz,
                                    make_float2(ix, iy), make_float2(dx, dy));
                } else {
                    za0.x = adj_cell(pz0.y, pw, pzm.x, pzp.x, pz0.x, z10.x, zz.x, ix, dx);
                    za0.y = adj_cell(pe, pz0.x, pzm.y, pzp.y, pz0.y, z10.y, zz.y, iy, dy);
                }
            }
        }
        const float2 pa0 = PACK ? pk_mul(c0, za0) : mul2(c0, za0);
        // ---- second step: z(kz-1) at row r-1, correlation of both steps at row r-1
        const int rb = r - 1;
        {
            // every lane joins the shuffles
            const float pw = __shfl_up_sync(FULL, pam.y, 1), pe = __shfl_down_sync(FULL, pam.x, 1);
            const float uaw = __shfl_up_sync(FULL, uam.y, 1), uae = __shfl_down_sync(FULL, uam.x, 1);
            const float ubw = __shfl_up_sync(FULL, ubm.y, 1), ube = __shfl_down_sync(FULL, ubm.x, 1);
            if (own && rb >= y0 && rb < ny) {
                const int rowb = rb * nx;
                const int dr = edge_dist(rb, ny);
                const float drow = dr < g.sponge_w ? g.damp[dr] : 1.f;
                float dx = drow, dy = drow;
                if (edge_x) { dx = damp_at(g, dca, dr); dy = damp_at(g, dcb, dr); }
                float ix = 0.f, iy = 0.f;
                if (rcvm) {
                    ix = ridm.x >= 0 ? rrb[ridm.x] : 0.f;
                    iy = ridm.y >= 0 ? rrb[ridm.y] : 0.f;
                }
                float2 cr = PF ? crm : *reinterpret_cast<const float2*>(corr + rowb + i);
                float2 zbv;
                if constexpr (PACK) {
                    zbv = adj_cell2(make_float2(pam.y, pe), make_float2(pw, pam.x), pam2, pa0, pam, zam, z1m,
                                    make_float2(ix, iy), make_float2(dx, dy));
                    const float2 la = lap5_2(make_float2(uam.y, uae), make_float2(uaw, uam.x), uam2, ua0, uam);
                    const float2 lb = lap5_2(make_float2(ubm.y, ube), make_float2(ubw, ubm.x), ubm2, ub0, ubm);
                    cr = pk_fma(zam, la, cr);
                    cr = pk_fma(zbv, lb, cr);
                } else {
                    zbv.x = adj_cell(pam.y, pw, pam2.x, pa0.x, pam.x, zam.x, z1m.x, ix, dx);
                    zbv.y = adj_cell(pe, pam.x, pam2.y, pa0.y, pam.y, zam.y, z1m.y, iy, dy);
                    const float lax = lap5(uam.y, uaw, uam2.x, ua0.x, uam.x);
                    const float lay = lap5(uae, uam.x, uam2.y, ua0.y, uam.y);
                    const float lbx = lap5(ubm.y, ubw, ubm2.x, ub0.x, ubm.x);
                    const float lby = lap5(ube, ubm.x, ubm2.y, ub0.y, ubm.y);
                    cr.x = __fmaf_rn(zam.x, lax, cr.x);
                    cr.y = __fmaf_rn(zam.y, lay, cr.y);
                    cr.x = __fmaf_rn(zbv.x, lbx, cr.x);
                    cr.y = __fmaf_rn(zbv.y, lby, cr.y);
                }
                *reinterpret_cast<float2*>(corr + rowb + i) = cr;
                *reinterpret_cast<float2*>(za + rowb + i) = zam;
                *reinterpret_cast<float2*>(zb + rowb + i) = zbv;
            }
        }
        z1m = z10; z10 = z1p;
        pzm = pz0; pz0 = pzp;
        c0 = cp;
        zam = za0;
        pam2 = pam; pam = pa0;
        uam2 = uam; uam = ua0;
        ubm2 = ubm; ubm = ub0;
        ridm = rid;
        rcvm = rcv;
        crm = cr_next;
    }
}

// AHEAD: 0 reads each row's inputs in the iteration that uses them; 1 also reads the
// correlation row one iteration ahead; 2 reads every input one iteration ahead (more loads in
// flight per warp).  SPLIT: warps whose strip lies inside the grid take a path without bounds
// predicates (the compiler then overlaps more loads, at more registers).  Minimum resident
// blocks per SM: 8 / 7 / 5 (AHEAD 0 / 1 / 2), 6 / 5 / 4 with SPLIT, one fewer with PACK.
constexpr int adj2_min_blocks(int ahead, bool split, bool pack) {
    return (split ? (ahead == 2 ? 4 : 6 - ahead) : (ahead == 2 ? 5 : 8 - ahead)) - (pack ? 1 : 0);
}

// PACK: the cell arithmetic in packed FP32x2 instructions (same bits, fewer instructions, register
// pairs).
template <int R, int AHEAD, bool SPLIT, bool PACK = false>
__global__ void __launch_bounds__(WARPS * 32, adj2_min_blocks(AHEAD, SPLIT, PACK))
    k_adj2_strip(DevGeo g, const float* __restrict__ coef, Adj2Step s) {
    const int warp = threadIdx.x >> 5;
    const int x0 = blockIdx.x * 60 - 2;
    const int y0 = (blockIdx.y * WARPS + warp) * R;
    if (y0 >= g.ny) return;
    if (SPLIT && x0 > 0 && x0 + 64 < g.nx && y0 >= 2 && y0 + R + 2 < g.ny)
        adj2_rows<R, AHEAD, false, PACK>(g, coef, s, x0, y0);
    else
        adj2_rows<R, AHEAD, true, PACK>(g, coef, s, x0, y0);
}

template <int R, int AHEAD, bool SPLIT, bool PACK = false>
void adj2_strip(const DevGeo& g, const float* coef, const Adj2Step& s, cudaStream_t st) {
    const int rows_per_block = WARPS * R;
    dim3 grid((g.nx + 59) / 60, (g.ny + rows_per_block - 1) / rows_per_block, s.ng);
    k_adj2_strip<R, AHEAD, SPLIT, PACK><<<grid, WARPS * 32, 0, st>>>(g, coef, s);
}

// ---------------------------------------------------------------------------
// Two adjoint steps per launch with four cells per lane (float4): 128-cell strips overlapping
// by one lane (4 cells) on each side, lanes 1..30 (120 cells) write.  Rows, rolling state,
// halo argument and arithmetic are those of k_adj2_strip, so the results are identical.
__device__ __forceinline__ float c4(const float4& v, int t) { return t == 0 ? v.x : t == 1 ? v.y : t == 2 ? v.z : v.w; }
__device__ __forceinline__ int c4(const int4& v, int t) { return t == 0 ? v.x : t == 1 ? v.y : t == 2 ? v.z : v.w; }

template <int R>
__global__ void __launch_bounds__(WARPS * 32, 4) k_adj2q_strip(DevGeo g, const float* __restrict__ coef, Adj2Step s) {
    const int nx = g.nx, ny = g.ny;
    const int gl = blockIdx.z;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x0 = blockIdx.x * 120 - 4;
    const int i = x0 + 4 * lane;
    const int y0 = (blockIdx.y * WARPS + warp) * R;
    if (y0 >= ny) return;
    const bool in = i >= 0 && i < nx;
    const bool own = in && lane >= 1 && lane <= 30;
    const float* z1 = s.z1 + gl * s.zstride;
    const float* z2 = s.z2 + gl * s.zstride;
    float* za = s.za + gl * s.zstride;
    float* zb = s.zb + gl * s.zstride;
    const float* ua = s.ua + gl * s.ustride;
    const float* ub = s.ub + gl * s.ustride;
    const float* rra = s.rra + gl * s.rrstride;
    const float* rrb = s.rrb + gl * s.rrstride;
    float* corr = s.corr + gl * s.cstride;
    const bool edge_x = x0 < g.sponge_w || x0 + 128 > nx - g.sponge_w;
    auto row_ok = [&](int r) { return in && r >= 0 && r < ny; };
    const RcvMask rk = rcv_mask(g, x0, x0 + 128);
    int dc[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) dc[t] = edge_dist(i + t, nx);
    // rolling state at the top of iteration r, as in k_adj2_strip
    float4 z1m = ld4(z1, (y0 - 2) * nx + i, row_ok(y0 - 2));
    float4 z10 = ld4(z1, (y0 - 1) * nx + i, row_ok(y0 - 1));
    float4 pzm = mul4(ld4(coef, (y0 - 2) * nx + i, row_ok(y0 - 2)), z1m);
    float4 c0 = ld4(coef, (y0 - 1) * nx + i, row_ok(y0 - 1));
    float4 pz0 = mul4(c0, z10);
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 zam = zero, pam2 = zero, pam = zero, uam2 = zero, uam = zero, ubm2 = zero, ubm = zero;
    int4 ridm = make_int4(-1, -1, -1, -1);
    bool rcvm = false;
#pragma unroll 1
    for (int r = y0 - 1; r <= y0 + R; ++r) {
        if (r > ny) break;
        const int row = r * nx;
        const bool ok = row_ok(r), okn = row_ok(r + 1);
        const float4 z1p = ld4(z1, row + nx + i, okn);
        const float4 cp = ld4(coef, row + nx + i, okn);
        const float4 zz = ld4(z2, row + i, ok);
        const float4 ua0 = ld4(ua, row + i, ok);
        const float4 ub0 = ld4(ub, row + i, ok);
        const bool rcv = rcv_row(g, rk, r);
        int4 rid = make_int4(-1, -1, -1, -1);
        if (rcv && ok) rid = *reinterpret_cast<const int4*>(g.rid + row + i);
        const float4 pzp = mul4(cp, z1p);
        // ---- first step: z(kz) at row r (all lanes; zero outside the grid; the halo cells
        // x0 .. x0+2 and x0+125 .. x0+127 are not read by any owned cell's second step)
        float4 za0 = zero;
        {
            const float pw = __shfl_up_sync(FULL, pz0.w, 1), pe = __shfl_down_sync(FULL, pz0.x, 1);
            if (ok) {
                const int dr = edge_dist(r, ny);
                const float drow = dr < g.sponge_w ? g.damp[dr] : 1.f;
                float v[4];
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const float d = edge_x ? damp_at(g, dc[t], dr) : drow;
                    const int id = c4(rid, t);
                    const float inj = (rcv && id >= 0) ? rra[id] : 0.f;
                    const float e = t < 3 ? c4(pz0, t + 1) : pe;
                    const float w = t > 0 ? c4(pz0, t - 1) : pw;
                    v[t] = adj_cell(e, w, c4(pzm, t), c4(pzp, t), c4(pz0, t), c4(z10, t), c4(zz, t), inj, d);
                }
                za0 = make_float4(v[0], v[1], v[2], v[3]);
            }
        }
        const float4 pa0 = mul4(c0, za0);
        // ---- second step: z(kz-1) at row r-1, correlation of both steps at row r-1
        const int rb = r - 1;
        {
            const float pw = __shfl_up_sync(FULL, pam.w, 1), pe = __shfl_down_sync(FULL, pam.x, 1);
            const float uaw = __shfl_up_sync(FULL, uam.w, 1), uae = __shfl_down_sync(FULL, uam.x, 1);
            const float ubw = __shfl_up_sync(FULL, ubm.w, 1), ube = __shfl_down_sync(FULL, ubm.x, 1);
            if (own && rb >= y0 && rb < ny) {
                const int rowb = rb * nx;
                const int dr = edge_dist(rb, ny);
                const float drow = dr < g.sponge_w ? g.damp[dr] : 1.f;
                float4 cr = *reinterpret_cast<const float4*>(corr + rowb + i);
                float zv[4], cv[4];
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const float d = edge_x ? damp_at(g, dc[t], dr) : drow;
                    const int id = c4(ridm, t);
                    const float inj = (rcvm && id >= 0) ? rrb[id] : 0.f;
                    const float e = t < 3 ? c4(pam, t + 1) : pe;
                    const float w = t > 0 ? c4(pam, t - 1) : pw;
                    zv[t] = adj_cell(e, w, c4(pam2, t), c4(pa0, t), c4(pam, t), c4(zam, t), c4(z1m, t), inj, d);
                    const float la = lap5(t < 3 ? c4(uam, t + 1) : uae, t > 0 ? c4(uam, t - 1) : uaw, c4(uam2, t),
                                          c4(ua0, t), c4(uam, t));
                    const float lb = lap5(t < 3 ? c4(ubm, t + 1) : ube, t > 0 ? c4(ubm, t - 1) : ubw, c4(ubm2, t),
                                          c4(ub0, t), c4(ubm, t));
                    cv[t] = __fmaf_rn(zv[t], lb, __fmaf_rn(c4(zam, t), la, c4(cr, t)));
                }
                *reinterpret_cast<float4*>(corr + rowb + i) = make_float4(cv[0], cv[1], cv[2], cv[3]);
                *reinterpret_cast<float4*>(za + rowb + i) = zam;
                *reinterpret_cast<float4*>(zb + rowb + i) = make_float4(zv[0], zv[1], zv[2], zv[3]);
            }
        }
        z1m = z10; z10 = z1p;
        pzm = pz0; pz0 = pzp;
        c0 = cp;
        zam = za0;
        pam2 = pam; pam = pa0;
        uam2 = uam; uam = ua0;
        ubm2 = ubm; ubm = ub0;
        ridm = rid;
        rcvm = rcv;
    }
}

template <int R>
void adj2q_strip(const DevGeo& g, const float* coef, const Adj2Step& s, cudaStream_t st) {
    const int rows_per_block = WARPS * R;
    dim3 grid((g.nx + 119) / 120, (g.ny + rows_per_block - 1) / rows_per_block, s.ng);
    k_adj2q_strip<R><<<grid, WARPS * 32, 0, st>>>(g, coef, s);
}

// ---------------------------------------------------------------------------
// Two adjoint steps per launch with the row inputs staged in shared memory: each warp keeps a
// ring of D rows of z(kz+1) and the coefficient (row r+1), z(kz+2), u(q), u(q-1) and the
// correlation (row r), filled by cp.async (16-byte copies, L2 only) D rows ahead of use, so
// the loads in flight do not cost registers.  Strips start at x0 = 60 bx - 4, 16-byte
// aligned, 64 cells wide, lanes 1..30 (60 cells) write; chunks outside the grid are
// zero-filled.  The cell arithmetic is that of k_adj2_strip, so the results are identical.
constexpr int ST_ARR = 6;                       // staged arrays per row
constexpr int ST_ROW = ST_ARR * 64;             // floats per staged row


// MB: minimum resident blocks per SM for the register allocator (7: 72 registers; 8: 64, one
// wave of C2's 1152 blocks, at the price of a few spilled values).
// UNR: the row loop fully unrolled (ring slots and the receiver-bit shift become constants).
// PK: a lane's two cells in packed FP32x2 instructions (adj_cell2, lap5_2, pk_fma: the same
// operation order and rounding, so the same bits, in fewer instructions).
template <int R, int D, int MB = 7, bool UNR = false, bool PK = false>
__global__ void __launch_bounds__(WARPS * 32, MB) k_adj2s_strip(DevGeo g, const float* __restrict__ coef, Adj2Step s) {
    extern __shared__ float4 st_mem4[];
    const int nx = g.nx, ny = g.ny;
    const int gl = blockIdx.z;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x0 = blockIdx.x * 60 - 4;
    const int i = x0 + 2 * lane;
    const int y0 = (blockIdx.y * WARPS + warp) * R;
    if (y0 >= ny) return;
    float* ring = reinterpret_cast<float*>(st_mem4) + warp * D * ST_ROW;
    const bool in = i >= 0 && i < nx;
    const bool own = in && lane >= 1 && lane <= 30;
    const int yend = min(y0 + R, ny);
    const float* z1 = s.z1 + gl * s.zstride;
    const float* z2 = s.z2 + gl * s.zstride;
    float* za = s.za + gl * s.zstride;
    float* zb = s.zb + gl * s.zstride;
    const float* ua = s.ua + gl * s.ustride;
    const float* ub = s.ub + gl * s.ustride;
    const float* rra = s.rra + gl * s.rrstride;
    const float* rrb = s.rrb + gl * s.rrstride;
    float* corr = s.corr + gl * s.cstride;
    const bool edge_x = x0 < g.sponge_w || x0 + 64 > nx - g.sponge_w;
    // any row y0-1 .. y0+R inside the sponge: only then do rows need the sponge table
    const bool damp_any = edge_x || y0 - 1 < g.sponge_w || y0 + R >= ny - g.sponge_w;
    auto row_ok = [&](int r) { return in && r >= 0 && r < ny; };
    const RcvMask rk = rcv_mask(g, x0, x0 + 64);
    // receiver flags of the warp's rows y0-1 .. y0+R (R + 2 <= 64): lane l tests rows y0-1+l and
    // y0+31+l, one ballot each, so the row loop reads a bit instead of the bitmap
    const unsigned rb_lo = __ballot_sync(FULL, rcv_row(g, rk, y0 - 1 + lane));
    const unsigned rb_hi = R + 2 > 32 ? __ballot_sync(FULL, rcv_row(g, rk, y0 + 31 + lane)) : 0u;
    const unsigned long long rbits = ((unsigned long long)rb_hi << 32) | rb_lo;
    const int dca = edge_dist(i, nx), dcb = edge_dist(i + 1, nx);
    // copy duty of this lane: chunk (lane & 15) of arrays 2*slot + (lane >> 4), slot 0..2
    const int ch = lane & 15, half = lane >> 4;
    const int cx = x0 + 4 * ch;                          // first cell of the chunk
    const bool cx_ok = cx >= 0 && cx + 3 < nx;           // nx % 4 == 0: chunks are all in or all out
    // staged arrays: 0 z1(t+1), 1 coef(t+1), 2 z2(t), 3 ua(t), 4 ub(t), 5 corr(t); lanes 0-15
    // copy arrays 0, 2, 4 and lanes 16-31 arrays 1, 3, 5, so each lane holds three sources
    const float* srcA = half ? coef : z1;               // row t+1
    const float* srcB = half ? ua : z2;                 // row t
    const float* srcC = half ? corr : ub;               // row t
    // shared-memory byte address of this lane's copy target in slot 0
    const unsigned ring_s = (unsigned)__cvta_generic_to_shared(ring) + 4u * (unsigned)(half * 64 + 4 * ch);
    auto stage = [&](int t, int slot) {                 // row t of the schedule into `slot`
        const unsigned dst = ring_s + 4u * (unsigned)(slot * ST_ROW);
        const bool r1 = cx_ok && t + 1 >= 0 && t + 1 < ny, r0 = cx_ok && t >= 0 && t < ny;
        const int o0 = t * nx + cx;
        cp_async16(dst, srcA + (r1 ? o0 + nx : 0), r1);
        cp_async16(dst + 4u * 2 * 64, srcB + (r0 ? o0 : 0), r0);
        cp_async16(dst + 4u * 4 * 64, srcC + (r0 ? o0 : 0), r0);
    };
    float2 z1m = ld2(z1, (y0 - 2) * nx + i, row_ok(y0 - 2));
    float2 z10 = ld2(z1, (y0 - 1) * nx + i, row_ok(y0 - 1));
    float2 pzm = mul2(ld2(coef, (y0 - 2) * nx + i, row_ok(y0 - 2)), z1m);
    float2 c0 = ld2(coef, (y0 - 1) * nx + i, row_ok(y0 - 1));
    float2 pz0 = mul2(c0, z10);
    float2 zam = make_float2(0.f, 0.f), pam2 = make_float2(0.f, 0.f), pam = make_float2(0.f, 0.f);
    float2 uam2 = make_float2(0.f, 0.f), uam = make_float2(0.f, 0.f);
    float2 ubm2 = make_float2(0.f, 0.f), ubm = make_float2(0.f, 0.f);
    float2 crm = make_float2(0.f, 0.f);
    int2 ridm = make_int2(-1, -1);
    bool rcvm = false;
    const int rlast = min(y0 + R, ny);                   // the loop covers rows y0-1 .. rlast
    // row y0-1 goes to slot 0, row y0-1+t to slot t mod D
#pragma unroll
    for (int t = 0; t < D; ++t) {                        // prologue: rows y0-1 .. y0+D-2
        if (y0 - 1 + t <= rlast) stage(y0 - 1 + t, t);
        cp_async_commit();
    }
    constexpr int UNROLL = UNR ? R + 2 : 1;
#pragma unroll UNROLL
    for (int t = 0; t < R + 2; ++t) {
        const int r = y0 - 1 + t;
        if (r > rlast) break;
        const int slot = t % D;                          // slot of row r
        const int row = r * nx;
        const bool ok = row_ok(r);
        cp_async_wait<D - 1>();                          // this lane's copies of row r are done
        __syncwarp();                                    // ... and every lane's
        const float* sr = ring + slot * ST_ROW + 2 * lane;
        const float2 z1p = *reinterpret_cast<const float2*>(sr + 0 * 64);
        const float2 cp = *reinterpret_cast<const float2*>(sr + 1 * 64);
        const float2 zz = *reinterpret_cast<const float2*>(sr + 2 * 64);
        const float2 ua0 = *reinterpret_cast<const float2*>(sr + 3 * 64);
        const float2 ub0 = *reinterpret_cast<const float2*>(sr + 4 * 64);
        const float2 cr_next = *reinterpret_cast<const float2*>(sr + 5 * 64);
        __syncwarp();                                    // the slot is free for row r+D
        if (r + D <= rlast) stage(r + D, slot);
        cp_async_commit();
        const bool rcv = (rbits >> t) & 1ull;
        int2 rid = make_int2(-1, -1);
        if (rcv && ok) rid = *reinterpret_cast<const int2*>(g.rid + row + i);
        const float2 pzp = PK ? pk_mul(cp, z1p) : mul2(cp, z1p);
        float2 za0 = make_float2(0.f, 0.f);
        {
            const float pw = __shfl_up_sync(FULL, pz0.y, 1), pe = __shfl_down_sync(FULL, pz0.x, 1);
            if (ok) {
                float dx = 1.f, dy = 1.f;
                if (damp_any) {
                    const int dr = edge_dist(r, ny);
                    const float drow = dr < g.sponge_w ? g.damp[dr] : 1.f;
                    dx = drow; dy = drow;
                    if (edge_x) { dx = damp_at(g, dca, dr); dy = damp_at(g, dcb, dr); }
                }
                float ix = 0.f, iy = 0.f;
                if (rcv) {
                    ix = rid.x >= 0 ? rra[rid.x] : 0.f;
                    iy = rid.y >= 0 ? rra[rid.y] : 0.f;
                }
                if constexpr (PK) {
                    za0 = adj_cell2(make_float2(pz0.y, pe), make_float2(pw, pz0.x), pzm, pzp, pz0, z10, zz,
                                    make_float2(ix, iy), make_float2(dx, dy));
                } else {
                    za0.x = adj_cell(pz0.y, pw, pzm.x, pzp.x, pz0.x, z10.x, zz.x, ix, dx);
                    za0.y = adj_cell(pe, pz0.x, pzm.y, pzp.y, pz0.y, z10.y, zz.y, iy, dy);
                }
            }
        }
        const float2 pa0 = PK ? pk_mul(c0, za0) : mul2(c0, za0);
        const int rb = r - 1;
        {
            const float pw = __shfl_up_sync(FULL, pam.y, 1), pe = __shfl_down_sync(FULL, pam.x, 1);
            const float uaw = __shfl_up_sync(FULL, uam.y, 1), uae = __shfl_down_sync(FULL, uam.x, 1);
            const float ubw = __shfl_up_sync(FULL, ubm.y, 1), ube = __shfl_down_sync(FULL, ubm.x, 1);
            if (own && rb >= y0 && rb < ny) {
                const int rowb = rb * nx;
                float dx = 1.f, dy = 1.f;
                if (damp_any) {
                    const int dr = edge_dist(rb, ny);
                    const float drow = dr < g.sponge_w ? g.damp[dr] : 1.f;
                    dx = drow; dy = drow;
                    if (edge_x) { dx = damp_at(g, dca, dr); dy = damp_at(g, dcb, dr); }
                }
                float ix = 0.f, iy = 0.f;
                if (rcvm) {
                    ix = ridm.x >= 0 ? rrb[ridm.x] : 0.f;
                    iy = ridm.y >= 0 ? rrb[ridm.y] : 0.f;
                }
                float2 zbv, cr = crm;
                if constexpr (PK) {
                    zbv = adj_cell2(make_float2(pam.y, pe), make_float2(pw, pam.x), pam2, pa0, pam, zam, z1m,
                                    make_float2(ix, iy), make_float2(dx, dy));
                    const float2 la = lap5_2(make_float2(uam.y, uae), make_float2(uaw, uam.x), uam2, ua0, uam);
                    const float2 lb = lap5_2(make_float2(ubm.y, ube), make_float2(ubw, ubm.x), ubm2, ub0, ubm);
                    cr = pk_fma(zam, la, cr);
                    cr = pk_fma(zbv, lb, cr);
                } else {
                    zbv.x = adj_cell(pam.y, pw, pam2.x, pa0.x, pam.x, zam.x, z1m.x, ix, dx);
                    zbv.y = adj_cell(pe, pam.x, pam2.y, pa0.y, pam.y, zam.y, z1m.y, iy, dy);
                    const float lax = lap5(uam.y, uaw, uam2.x, ua0.x, uam.x);
                    const float lay = lap5(uae, uam.x, uam2.y, ua0.y, uam.y);
                    const float lbx = lap5(ubm.y, ubw, ubm2.x, ub0.x, ubm.x);
                    const float lby = lap5(ube, ubm.x, ubm2.y, ub0.y, ubm.y);
                    cr.x = __fmaf_rn(zam.x, lax, cr.x);
                    cr.y = __fmaf_rn(zam.y, lay, cr.y);
                    cr.x = __fmaf_rn(zbv.x, lbx, cr.x);
                    cr.y = __fmaf_rn(zbv.y, lby, cr.y);
                }
                *reinterpret_cast<float2*>(corr + rowb + i) = cr;
                *reinterpret_cast<float2*>(za + rowb + i) = zam;
                *reinterpret_cast<float2*>(zb + rowb + i) = zbv;
            }
        }
        z1m = z10; z10 = z1p;
        pzm = pz0; pz0 = pzp;
        c0 = cp;
        zam = za0;
        pam2 = pam; pam = pa0;
        uam2 = uam; uam = ua0;
        ubm2 = ubm; ubm = ub0;
        ridm = rid;
        rcvm = rcv;
        crm = cr_next;
    }
    cp_async_wait<0>();                                  // nothing left in flight at exit
}

template <int R, int D, int MB = 7, bool UNR = false, bool PK = false>
void adj2s_strip(const DevGeo& g, const float* coef, const Adj2Step& s, cudaStream_t st) {
    const int rows_per_block = WARPS * R;
    const size_t smem = sizeof(float) * WARPS * D * ST_ROW;
    dim3 grid((g.nx + 2 + 59) / 60, (g.ny + rows_per_block - 1) / rows_per_block, s.ng);
    k_adj2s_strip<R, D, MB, UNR, PK><<<grid, WARPS * 32, smem, st>>>(g, coef, s);
}

// ---------------------------------------------------------------------------
// Two adjoint steps per launch, staged, four cells per lane: 128-cell strips overlapping by one
// lane (4 cells) on each side (lanes 1..30 write 120 cells), the row inputs in a per-warp
// shared-memory ring of D rows filled by cp.async (each lane copies one 16-byte chunk of each
// of the six arrays per row), the sponge factor from the per-cell map (read one row ahead), the
// row loop fully unrolled.  Rolling state and cell arithmetic are those of k_adj2_strip, so the
// results are identical.
constexpr int S4_ROW = ST_ARR * 128;           // floats per staged row (six arrays of 128 cells)

template <int R, int D, int MB>
__global__ void __launch_bounds__(WARPS * 32, MB) k_adj2s4_strip(DevGeo g, const float* __restrict__ coef, Adj2Step s) {
    extern __shared__ float4 st_mem4[];
    const int nx = g.nx, ny = g.ny;
    const int gl = blockIdx.z;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x0 = blockIdx.x * 120 - 4;
    const int i = x0 + 4 * lane;
    const int y0 = (blockIdx.y * WARPS + warp) * R;
    if (y0 >= ny) return;
    float* ring = reinterpret_cast<float*>(st_mem4) + warp * D * S4_ROW;
    const bool in = i >= 0 && i < nx;                // nx % 4 == 0: a lane's chunk is all in or out
    const bool own = in && lane >= 1 && lane <= 30;
    const float* z1 = s.z1 + gl * s.zstride;
    const float* z2 = s.z2 + gl * s.zstride;
    float* za = s.za + gl * s.zstride;
    float* zb = s.zb + gl * s.zstride;
    const float* ua = s.ua + gl * s.ustride;
    const float* ub = s.ub + gl * s.ustride;
    const float* rra = s.rra + gl * s.rrstride;
    const float* rrb = s.rrb + gl * s.rrstride;
    float* corr = s.corr + gl * s.cstride;
    const float* dmap = g.dmap;
    auto row_ok = [&](int r) { return in && r >= 0 && r < ny; };
    const RcvMask rk = rcv_mask(g, x0, x0 + 128);
    const unsigned rb_lo = __ballot_sync(FULL, rcv_row(g, rk, y0 - 1 + lane));
    const unsigned rb_hi = R + 2 > 32 ? __ballot_sync(FULL, rcv_row(g, rk, y0 + 31 + lane)) : 0u;
    const unsigned long long rbits = ((unsigned long long)rb_hi << 32) | rb_lo;
    // staged arrays: 0 z1(t+1), 1 coef(t+1), 2 z2(t), 3 ua(t), 4 ub(t), 5 corr(t); lane copies its chunk
    const unsigned ring_s = (unsigned)__cvta_generic_to_shared(ring) + 16u * (unsigned)lane;
    auto stage = [&](int t, int slot) {                 // row t of the schedule into `slot`
        const unsigned dst = ring_s + 4u * (unsigned)(slot * S4_ROW);
        const bool r1 = row_ok(t + 1), r0 = row_ok(t);
        const int o0 = t * nx + i;
        cp_async16(dst + 4u * 0 * 128, z1 + (r1 ? o0 + nx : 0), r1);
        cp_async16(dst + 4u * 1 * 128, coef + (r1 ? o0 + nx : 0), r1);
        cp_async16(dst + 4u * 2 * 128, z2 + (r0 ? o0 : 0), r0);
        cp_async16(dst + 4u * 3 * 128, ua + (r0 ? o0 : 0), r0);
        cp_async16(dst + 4u * 4 * 128, ub + (r0 ? o0 : 0), r0);
        cp_async16(dst + 4u * 5 * 128, corr + (r0 ? o0 : 0), r0);
    };
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    int o = (y0 - 1) * nx;
    float4 z1m = ld4(z1, o - nx + i, row_ok(y0 - 2));
    float4 z10 = ld4(z1, o + i, row_ok(y0 - 1));
    float4 pzm = mul4(ld4(coef, o - nx + i, row_ok(y0 - 2)), z1m);
    float4 c0 = ld4(coef, o + i, row_ok(y0 - 1));
    float4 pz0 = mul4(c0, z10);
    float4 zam = zero, pam2 = zero, pam = zero, uam2 = zero, uam = zero, ubm2 = zero, ubm = zero, crm = zero;
    float4 dm = zero;
    float4 d0 = ld4(dmap, o + i, row_ok(y0 - 1));       // sponge of row r, read one row ahead
    int4 ridm = make_int4(-1, -1, -1, -1);
    bool rcvm = false;
    const int rlast = min(y0 + R, ny);
#pragma unroll
    for (int t = 0; t < D; ++t) {                        // prologue: rows y0-1 .. y0+D-2
        if (y0 - 1 + t <= rlast) stage(y0 - 1 + t, t);
        cp_async_commit();
    }
#pragma unroll
    for (int t = 0; t < R + 2; ++t) {
        const int r = y0 - 1 + t;
        if (r > rlast) break;
        const int slot = t % D;
        const bool ok = row_ok(r);
        cp_async_wait<D - 1>();
        __syncwarp();
        const float* sr = ring + slot * S4_ROW + 4 * lane;
        const float4 z1p = *reinterpret_cast<const float4*>(sr + 0 * 128);
        const float4 cp = *reinterpret_cast<const float4*>(sr + 1 * 128);
        const float4 zz = *reinterpret_cast<const float4*>(sr + 2 * 128);
        const float4 ua0 = *reinterpret_cast<const float4*>(sr + 3 * 128);
        const float4 ub0 = *reinterpret_cast<const float4*>(sr + 4 * 128);
        const float4 cr_next = *reinterpret_cast<const float4*>(sr + 5 * 128);
        __syncwarp();
        if (r + D <= rlast) stage(r + D, slot);
        cp_async_commit();
        const float4 d1 = ld4(dmap, o + nx + i, row_ok(r + 1));   // next row's sponge
        const bool rcv = (rbits >> t) & 1ull;
        int4 rid = make_int4(-1, -1, -1, -1);
        if (rcv && ok) rid = *reinterpret_cast<const int4*>(g.rid + o + i);
        const float4 pzp = mul4(cp, z1p);
        float4 za0 = zero;
        {
            const float pw = __shfl_up_sync(FULL, pz0.w, 1), pe = __shfl_down_sync(FULL, pz0.x, 1);
            if (ok) {
                float4 inj = zero;
                if (rcv) {
                    inj.x = rid.x >= 0 ? rra[rid.x] : 0.f;
                    inj.y = rid.y >= 0 ? rra[rid.y] : 0.f;
                    inj.z = rid.z >= 0 ? rra[rid.z] : 0.f;
                    inj.w = rid.w >= 0 ? rra[rid.w] : 0.f;
                }
                za0.x = adj_cell(pz0.y, pw, pzm.x, pzp.x, pz0.x, z10.x, zz.x, inj.x, d0.x);
                za0.y = adj_cell(pz0.z, pz0.x, pzm.y, pzp.y, pz0.y, z10.y, zz.y, inj.y, d0.y);
                za0.z = adj_cell(pz0.w, pz0.y, pzm.z, pzp.z, pz0.z, z10.z, zz.z, inj.z, d0.z);
                za0.w = adj_cell(pe, pz0.z, pzm.w, pzp.w, pz0.w, z10.w, zz.w, inj.w, d0.w);
            }
        }
        const float4 pa0 = mul4(c0, za0);
        {
            const float pw = __shfl_up_sync(FULL, pam.w, 1), pe = __shfl_down_sync(FULL, pam.x, 1);
            const float uaw = __shfl_up_sync(FULL, uam.w, 1), uae = __shfl_down_sync(FULL, uam.x, 1);
            const float ubw = __shfl_up_sync(FULL, ubm.w, 1), ube = __shfl_down_sync(FULL, ubm.x, 1);
            if (t >= 2 && own && r - 1 < ny) {
                const int ob = o - nx;
                float4 inj = zero;
                if (rcvm) {
                    inj.x = ridm.x >= 0 ? rrb[ridm.x] : 0.f;
                    inj.y = ridm.y >= 0 ? rrb[ridm.y] : 0.f;
                    inj.z = ridm.z >= 0 ? rrb[ridm.z] : 0.f;
                    inj.w = ridm.w >= 0 ? rrb[ridm.w] : 0.f;
                }
                float4 zbv;
                zbv.x = adj_cell(pam.y, pw, pam2.x, pa0.x, pam.x, zam.x, z1m.x, inj.x, dm.x);
                zbv.y = adj_cell(pam.z, pam.x, pam2.y, pa0.y, pam.y, zam.y, z1m.y, inj.y, dm.y);
                zbv.z = adj_cell(pam.w, pam.y, pam2.z, pa0.z, pam.z, zam.z, z1m.z, inj.z, dm.z);
                zbv.w = adj_cell(pe, pam.z, pam2.w, pa0.w, pam.w, zam.w, z1m.w, inj.w, dm.w);
                float4 cr = crm;
                cr.x = __fmaf_rn(zam.x, lap5(uam.y, uaw, uam2.x, ua0.x, uam.x), cr.x);
                cr.y = __fmaf_rn(zam.y, lap5(uam.z, uam.x, uam2.y, ua0.y, uam.y), cr.y);
                cr.z = __fmaf_rn(zam.z, lap5(uam.w, uam.y, uam2.z, ua0.z, uam.z), cr.z);
                cr.w = __fmaf_rn(zam.w, lap5(uae, uam.z, uam2.w, ua0.w, uam.w), cr.w);
                cr.x = __fmaf_rn(zbv.x, lap5(ubm.y, ubw, ubm2.x, ub0.x, ubm.x), cr.x);
                cr.y = __fmaf_rn(zbv.y, lap5(ubm.z, ubm.x, ubm2.y, ub0.y, ubm.y), cr.y);
                cr.z = __fmaf_rn(zbv.z, lap5(ubm.w, ubm.y, ubm2.z, ub0.z, ubm.z), cr.z);
                cr.w = __fmaf_rn(zbv.w, lap5(ube, ubm.z, ubm2.w, ub0.w, ubm.w), cr.w);
                *reinterpret_cast<float4*>(corr + ob + i) = cr;
                *reinterpret_cast<float4*>(za + ob + i) = zam;
                *reinterpret_cast<float4*>(zb + ob + i) = zbv;
            }
        }
        z1m = z10; z10 = z1p;
        pzm = pz0; pz0 = pzp;
        c0 = cp;
        zam = za0;
        pam2 = pam; pam = pa0;
        uam2 = uam; uam = ua0;
        ubm2 = ubm; ubm = ub0;
        dm = d0; d0 = d1;
        ridm = rid;
        rcvm = rcv;
        crm = cr_next;
        o += nx;
    }
    cp_async_wait<0>();
}

template <int R, int D, int MB>
void adj2s4_strip(const DevGeo& g, const float* coef, const Adj2Step& s, cudaStream_t st) {
    const int rows_per_block = WARPS * R;
    const size_t smem = sizeof(float) * WARPS * D * S4_ROW;
    dim3 grid((g.nx + 119) / 120, (g.ny + rows_per_block - 1) / rows_per_block, s.ng);
    k_adj2s4_strip<R, D, MB><<<grid, WARPS * 32, smem, st>>>(g, coef, s);
}

// ---------------------------------------------------------------------------
// Two adjoint steps per launch, lean form: four cells per lane, 128-cell strips overlapping by
// one lane (4 cells) on each side (lanes 1..30, 120 cells, write; lanes 0 and 31 compute the
// first step as halo), rows y0-1 .. y0+R in a fully unrolled loop with every access predicated,
// the sponge factor from the per-cell map, receiver rows flagged by two ballots at kernel start.
// Rolling state and cell arithmetic are those of k_adj2_strip, so the results are identical.
template <int R, int MB>
__global__ void __launch_bounds__(WARPS * 32, MB) k_adjl2_strip(DevGeo g, const float* __restrict__ coef, Adj2Step s) {
    const int nx = g.nx, ny = g.ny;
    const int gl = blockIdx.z;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x0 = blockIdx.x * 120 - 4;
    const int i = x0 + 4 * lane;
    const int y0 = (blockIdx.y * WARPS + warp) * R;
    if (y0 >= ny) return;
    const bool in = i >= 0 && i < nx;                // nx % 4 == 0: a lane's four cells are all in or out
    const bool own = in && lane >= 1 && lane <= 30;
    const float* __restrict__ z1 = s.z1 + gl * s.zstride;
    const float* __restrict__ z2 = s.z2 + gl * s.zstride;
    float* __restrict__ za = s.za + gl * s.zstride;
    float* __restrict__ zb = s.zb + gl * s.zstride;
    const float* __restrict__ ua = s.ua + gl * s.ustride;
    const float* __restrict__ ub = s.ub + gl * s.ustride;
    const float* __restrict__ rra = s.rra + gl * s.rrstride;
    const float* __restrict__ rrb = s.rrb + gl * s.rrstride;
    float* __restrict__ corr = s.corr + gl * s.cstride;
    const float* __restrict__ dmap = g.dmap;
    // receiver flags of rows y0-1 .. y0+R (R + 2 <= 64)
    const RcvMask rk = rcv_mask(g, x0, x0 + STRIP);
    const unsigned rb_lo = __ballot_sync(FULL, rcv_row(g, rk, y0 - 1 + lane));
    const unsigned rb_hi = R + 2 > 32 ? __ballot_sync(FULL, rcv_row(g, rk, y0 + 31 + lane)) : 0u;
    const unsigned long long rbits = ((unsigned long long)rb_hi << 32) | rb_lo;
    auto row_in = [&](int r) { return in && r >= 0 && r < ny; };
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    // state at the top of iteration t (first step at row r = y0-1+t, second at row r-1):
    // z(kz+1) rows r-1, r; c z(kz+1) rows r-1, r; the coefficient row r; z(kz) row r-1 and
    // c z(kz) rows r-2, r-1; u(q), u(q-1) rows r-2, r-1; sponge and receivers of row r-1
    int o = (y0 - 1) * nx;                            // offset of row r (32-bit: nx*ny < 2^31)
    float4 z1m = ld4(z1, o - nx + i, row_in(y0 - 2));
    float4 z10 = ld4(z1, o + i, row_in(y0 - 1));
    float4 pzm = mul4(ld4(coef, o - nx + i, row_in(y0 - 2)), z1m);
    float4 c0 = ld4(coef, o + i, row_in(y0 - 1));
    float4 pz0 = mul4(c0, z10);
    float4 zam = zero, pam2 = zero, pam = zero, uam2 = zero, uam = zero, ubm2 = zero, ubm = zero, dm = zero;
    int4 ridm = make_int4(-1, -1, -1, -1);
    bool rcvm = false;
#pragma unroll
    for (int t = 0; t < R + 2; ++t) {
        const int r = y0 - 1 + t;
        if (r > ny) break;                            // uniform per warp
        const bool okr = row_in(r), okp = row_in(r + 1);
        const float4 z1p = ld4(z1, o + nx + i, okp);
        const float4 cp = ld4(coef, o + nx + i, okp);
        const float4 zz = ld4(z2, o + i, okr);
        const float4 ua0 = ld4(ua, o + i, okr);
        const float4 ub0 = ld4(ub, o + i, okr);
        const float4 d0 = ld4(dmap, o + i, okr);
        const bool rcv = (rbits >> t) & 1ull;
        int4 rid = make_int4(-1, -1, -1, -1);
        if (rcv && okr) rid = *reinterpret_cast<const int4*>(g.rid + o + i);
        const float4 pzp = mul4(cp, z1p);
        // ---- first step: z(kz) at row r (zero outside the grid)
        float4 za0 = zero;
        {
            const float pw = __shfl_up_sync(FULL, pz0.w, 1), pe = __shfl_down_sync(FULL, pz0.x, 1);
            if (okr) {
                float4 inj = zero;
                if (rcv) {
                    inj.x = rid.x >= 0 ? rra[rid.x] : 0.f;
                    inj.y = rid.y >= 0 ? rra[rid.y] : 0.f;
                    inj.z = rid.z >= 0 ? rra[rid.z] : 0.f;
                    inj.w = rid.w >= 0 ? rra[rid.w] : 0.f;
                }
                za0.x = adj_cell(pz0.y, pw, pzm.x, pzp.x, pz0.x, z10.x, zz.x, inj.x, d0.x);
                za0.y = adj_cell(pz0.z, pz0.x, pzm.y, pzp.y, pz0.y, z10.y, zz.y, inj.y, d0.y);
                za0.z = adj_cell(pz0.w, pz0.y, pzm.z, pzp.z, pz0.z, z10.z, zz.z, inj.z, d0.z);
                za0.w = adj_cell(pe, pz0.z, pzm.w, pzp.w, pz0.w, z10.w, zz.w, inj.w, d0.w);
            }
        }
        const float4 pa0 = mul4(c0, za0);
        // ---- second step: z(kz-1) at row r-1, correlation of both steps at row r-1
        {
            const float pw = __shfl_up_sync(FULL, pam.w, 1), pe = __shfl_down_sync(FULL, pam.x, 1);
            const float uaw = __shfl_up_sync(FULL, uam.w, 1), uae = __shfl_down_sync(FULL, uam.x, 1);
            const float ubw = __shfl_up_sync(FULL, ubm.w, 1), ube = __shfl_down_sync(FULL, ubm.x, 1);
            if (t >= 2 && own && r - 1 < ny) {
                const int ob = o - nx;
                float4 inj = zero;
                if (rcvm) {
                    inj.x = ridm.x >= 0 ? rrb[ridm.x] : 0.f;
                    inj.y = ridm.y >= 0 ? rrb[ridm.y] : 0.f;
                    inj.z = ridm.z >= 0 ? rrb[ridm.z] : 0.f;
                    inj.w = ridm.w >= 0 ? rrb[ridm.w] : 0.f;
                }
                float4 zbv;
                zbv.x = adj_cell(pam.y, pw, pam2.x, pa0.x, pam.x, zam.x, z1m.x, inj.x, dm.x);
                zbv.y = adj_cell(pam.z, pam.x, pam2.y, pa0.y, pam.y, zam.y, z1m.y, inj.y, dm.y);
                zbv.z = adj_cell(pam.w, pam.y, pam2.z, pa0.z, pam.z, zam.z, z1m.z, inj.z, dm.z);
                zbv.w = adj_cell(pe, pam.z, pam2.w, pa0.w, pam.w, zam.w, z1m.w, inj.w, dm.w);
                float4 cr = *reinterpret_cast<const float4*>(corr + ob + i);
                cr.x = __fmaf_rn(zam.x, lap5(uam.y, uaw, uam2.x, ua0.x, uam.x), cr.x);
                cr.y = __fmaf_rn(zam.y, lap5(uam.z, uam.x, uam2.y, ua0.y, uam.y), cr.y);
                cr.z = __fmaf_rn(zam.z, lap5(uam.w, uam.y, uam2.z, ua0.z, uam.z), cr.z);
                cr.w = __fmaf_rn(zam.w, lap5(uae, uam.z, uam2.w, ua0.w, uam.w), cr.w);
                cr.x = __fmaf_rn(zbv.x, lap5(ubm.y, ubw, ubm2.x, ub0.x, ubm.x), cr.x);
                cr.y = __fmaf_rn(zbv.y, lap5(ubm.z, ubm.x, ubm2.y, ub0.y, ubm.y), cr.y);
                cr.z = __fmaf_rn(zbv.z, lap5(ubm.w, ubm.y, ubm2.z, ub0.z, ubm.z), cr.z);
                cr.w = __fmaf_rn(zbv.w, lap5(ube, ubm.z, ubm2.w, ub0.w, ubm.w), cr.w);
                *reinterpret_cast<float4*>(corr + ob + i) = cr;
                *reinterpret_cast<float4*>(za + ob + i) = zam;
                *reinterpret_cast<float4*>(zb + ob + i) = zbv;
            }
        }
        z1m = z10; z10 = z1p;
        pzm = pz0; pz0 = pzp;
        c0 = cp;
        zam = za0;
        pam2 = pam; pam = pa0;
        uam2 = uam; uam = ua0;
        ubm2 = ubm; ubm = ub0;
        dm = d0;
        ridm = rid;
        rcvm = rcv;
        o += nx;
    }
}

template <int R, int MB>
void adjl2_strip(const DevGeo& g, const float* coef, const Adj2Step& s, cudaStream_t st) {
    const int rows_per_block = WARPS * R;
    dim3 grid((g.nx + 119) / 120, (g.ny + rows_per_block - 1) / rows_per_block, s.ng);
    k_adjl2_strip<R, MB><<<grid, WARPS * 32, 0, st>>>(g, coef, s);
}

// ---------------------------------------------------------------------------
// Two forward steps per launch.  Same strip geometry as k_adj2_strip (2 cells
// per lane, 64-cell strips overlapping by one lane each side, lanes 1..30
// write).  u(k+1) rows y0-1 .. y0+R roll through registers and u(k+2) follows
// one row behind, so u(k-1), u(k) and the coefficient are read once per two
// steps; both new slices are written (the next launch and the adjoint need
// them).  The gather blocks record the two input slices, which are complete.
struct Fwd2Step {
    const float* up;   // u(k-1)
    const float* uc;   // u(k)
    float* u1;         // u(k+1) out
    float* u2;         // u(k+2) out
    int64_t gstride;
    float* ck1;        // optional checkpoint copies of u(k+1), u(k+2) (pass-group 0)
    float* ck2;
    int64_t ckstride;
    int k, g0, ng;
    int gka, gkb;      // slices gathered from up (k-1) and uc (k); < 2: none
    const float* gmeas;
    float* gout;
};

__device__ __forceinline__ void gather_slice(const DevGeo& g, const float* u, int gl, int g0, int gk,
                                             const float* gmeas, float* gout) {
    const int64_t base = ((int64_t)gl * g.nt + gk) * g.nch;
    const bool noisy = gmeas && g.noise_key;
    const uint64_t key = noisy ? *g.noise_key : 0;
    for (int c = threadIdx.x; c < g.nch; c += blockDim.x) {
        const int cell = g.rcv[c];
        float v = cell >= 0 ? u[cell] : 0.f;
        if (noisy) v *= noise_factor(key, g.noise_level, g0 + gl, gk, c);
        gout[base + c] = gmeas ? (cell >= 0 ? gmeas[base + c] - v : 0.f) : v;
    }
}

template <int R>
__global__ void __launch_bounds__(WARPS * 32, 8) k_fwd2_strip(DevGeo g, const float* __restrict__ coef, Fwd2Step s) {
    const int nx = g.nx, ny = g.ny;
    const int gl = blockIdx.z;
    if (blockIdx.y == gridDim.y - 1) {
        if (blockIdx.x != 0) return;
        if (s.gka >= 2) gather_slice(g, s.up + gl * s.gstride, gl, s.g0, s.gka, s.gmeas, s.gout);
        if (s.gkb >= 2) gather_slice(g, s.uc + gl * s.gstride, gl, s.g0, s.gkb, s.gmeas, s.gout);
        return;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x0 = blockIdx.x * 60 - 2;
    const int i = x0 + 2 * lane;
    const int y0 = (blockIdx.y * WARPS + warp) * R;
    if (y0 >= ny) return;
    const bool in = i >= 0 && i < nx;
    const bool own = in && lane >= 1 && lane <= 30;
    const float* uc = s.uc + gl * s.gstride;
    const float* up = s.up + gl * s.gstride;
    float* u1 = s.u1 + gl * s.gstride;
    float* u2 = s.u2 + gl * s.gstride;
    float* ck1 = s.ck1 ? s.ck1 + gl * s.ckstride : nullptr;
    float* ck2 = s.ck2 ? s.ck2 + gl * s.ckstride : nullptr;
    const bool edge_x = x0 < g.sponge_w || x0 + 64 > nx - g.sponge_w;
    const int32_t* em = g.emit + (int64_t)(s.g0 + gl) * g.gs;
    const bool src1 = s.k < g.n_src_steps, src2 = s.k + 1 < g.n_src_steps;
    const float a1 = src1 ? g.src[s.k] : 0.f, a2 = src2 ? g.src[s.k + 1] : 0.f;
    auto row_ok = [&](int r) { return in && r >= 0 && r < ny; };
    float2 u0m = ld2(uc, (int64_t)(y0 - 2) * nx + i, row_ok(y0 - 2));
    float2 u00 = ld2(uc, (int64_t)(y0 - 1) * nx + i, row_ok(y0 - 1));
    float2 cm = ld2(coef, (int64_t)(y0 - 2) * nx + i, row_ok(y0 - 2));
    float2 v1m2 = make_float2(0.f, 0.f), v1m = make_float2(0.f, 0.f);
#pragma unroll 1
    for (int r = y0 - 1; r <= y0 + R; ++r) {
        if (r > ny) break;
        const int64_t row = (int64_t)r * nx;
        const bool ok = row_ok(r);
        const float2 u0p = ld2(uc, row + nx + i, row_ok(r + 1));
        const float2 p = ld2(up, row + i, ok);
        const float2 c0 = ld2(coef, row + i, ok);
        // ---- u(k+1) at row r, all lanes (zero outside the grid)
        float w = __shfl_up_sync(FULL, u00.y, 1), e = __shfl_down_sync(FULL, u00.x, 1);
        if (lane == 0) w = (ok && x0 > 0) ? uc[row + x0 - 1] : 0.f;
        if (lane == 31) e = (ok && x0 + 64 < nx) ? uc[row + x0 + 64] : 0.f;
        float2 v10 = make_float2(0.f, 0.f);
        if (ok) {
            const bool near = edge_x || r < g.sponge_w || r >= ny - g.sponge_w;
            const float dx = near ? sponge(g, i, r) : 1.f;
            const float dy = near ? sponge(g, i + 1, r) : 1.f;
            const float ax = src1 ? emit_at(em, g.gs, row + i, a1) : 0.f;
            const float ay = src1 ? emit_at(em, g.gs, row + i + 1, a1) : 0.f;
            v10.x = fwd_cell(u00.y, w, u0m.x, u0p.x, u00.x, p.x, c0.x, dx, ax);
            v10.y = fwd_cell(e, u00.x, u0m.y, u0p.y, u00.y, p.y, c0.y, dy, ay);
        }
        // ---- u(k+2) at row r-1
        const int rb = r - 1;
        const float w2 = __shfl_up_sync(FULL, v1m.y, 1), e2 = __shfl_down_sync(FULL, v1m.x, 1);
        if (own && rb >= y0 && rb < ny) {
            const int64_t rowb = (int64_t)rb * nx;
            const bool near = edge_x || rb < g.sponge_w || rb >= ny - g.sponge_w;
            const float dx = near ? sponge(g, i, rb) : 1.f;
            const float dy = near ? sponge(g, i + 1, rb) : 1.f;
            const float ax = src2 ? emit_at(em, g.gs, rowb + i, a2) : 0.f;
            const float ay = src2 ? emit_at(em, g.gs, rowb + i + 1, a2) : 0.f;
            float2 v2;
            v2.x = fwd_cell(v1m.y, w2, v1m2.x, v10.x, v1m.x, u0m.x, cm.x, dx, ax);
            v2.y = fwd_cell(e2, v1m.x, v1m2.y, v10.y, v1m.y, u0m.y, cm.y, dy, ay);
            *reinterpret_cast<float2*>(u1 + rowb + i) = v1m;
            *reinterpret_cast<float2*>(u2 + rowb + i) = v2;
            if (ck1) *reinterpret_cast<float2*>(ck1 + rowb + i) = v1m;
            if (ck2) *reinterpret_cast<float2*>(ck2 + rowb + i) = v2;
        }
        u0m = u00; u00 = u0p;
        cm = c0;
        v1m2 = v1m; v1m = v10;
    }
}

// Same two-step forward with four cells per lane: 128-cell strips overlapping
// by one lane (4 cells) on each side, lanes 1..30 (120 cells) write, 16-byte
// accesses.
__device__ __forceinline__ float4 fwd_row4(const float4& u, float w, float e, const float4& s, const float4& n,
                                           const float4& up, const float4& c, const float d[4], const float a[4]) {
    float4 v;
    v.x = fwd_cell(u.y, w, s.x, n.x, u.x, up.x, c.x, d[0], a[0]);
    v.y = fwd_cell(u.z, u.x, s.y, n.y, u.y, up.y, c.y, d[1], a[1]);
    v.z = fwd_cell(u.w, u.y, s.z, n.z, u.z, up.z, c.z, d[2], a[2]);
    v.w = fwd_cell(e, u.z, s.w, n.w, u.w, up.w, c.w, d[3], a[3]);
    return v;
}

template <int R>
__global__ void __launch_bounds__(WARPS * 32, 6) k_fwd2q_strip(DevGeo g, const float* __restrict__ coef, Fwd2Step s) {
    const int nx = g.nx, ny = g.ny;
    const int gl = blockIdx.z;
    if (blockIdx.y == gridDim.y - 1) {
        if (blockIdx.x != 0) return;
        if (s.gka >= 2) gather_slice(g, s.up + gl * s.gstride, gl, s.g0, s.gka, s.gmeas, s.gout);
        if (s.gkb >= 2) gather_slice(g, s.uc + gl * s.gstride, gl, s.g0, s.gkb, s.gmeas, s.gout);
        return;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x0 = blockIdx.x * 120 - 4;
    const int i = x0 + 4 * lane;
    const int y0 = (blockIdx.y * WARPS + warp) * R;
    if (y0 >= ny) return;
    const bool in = i >= 0 && i < nx;
    const bool own = in && lane >= 1 && lane <= 30;
    const float* uc = s.uc + gl * s.gstride;
    const float* up = s.up + gl * s.gstride;
    float* u1 = s.u1 + gl * s.gstride;
    float* u2 = s.u2 + gl * s.gstride;
    float* ck1 = s.ck1 ? s.ck1 + gl * s.ckstride : nullptr;
    float* ck2 = s.ck2 ? s.ck2 + gl * s.ckstride : nullptr;
    const bool edge_x = x0 < g.sponge_w || x0 + STRIP > nx - g.sponge_w;
    const int32_t* em = g.emit + (int64_t)(s.g0 + gl) * g.gs;
    const bool src1 = s.k < g.n_src_steps, src2 = s.k + 1 < g.n_src_steps;
    const float a1 = src1 ? g.src[s.k] : 0.f, a2 = src2 ? g.src[s.k + 1] : 0.f;
    auto row_ok = [&](int r) { return in && r >= 0 && r < ny; };
    auto factors = [&](int r, bool srcf, float amp, float d[4], float a[4]) {
        const bool near = edge_x || r < g.sponge_w || r >= ny - g.sponge_w;
        const int64_t q = (int64_t)r * nx + i;
        for (int t = 0; t < 4; ++t) {
            d[t] = near ? sponge(g, i + t, r) : 1.f;
            a[t] = srcf ? emit_at(em, g.gs, q + t, amp) : 0.f;
        }
    };
    float4 u0m = ld4(uc, (int64_t)(y0 - 2) * nx + i, row_ok(y0 - 2));
    float4 u00 = ld4(uc, (int64_t)(y0 - 1) * nx + i, row_ok(y0 - 1));
    float4 cm = ld4(coef, (int64_t)(y0 - 2) * nx + i, row_ok(y0 - 2));
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 v1m2 = zero4, v1m = zero4;
#pragma unroll 1
    for (int r = y0 - 1; r <= y0 + R; ++r) {
        if (r > ny) break;
        const int64_t row = (int64_t)r * nx;
        const bool ok = row_ok(r);
        const float4 u0p = ld4(uc, row + nx + i, row_ok(r + 1));
        const float4 p = ld4(up, row + i, ok);
        const float4 c0 = ld4(coef, row + i, ok);
        float w = __shfl_up_sync(FULL, u00.w, 1), e = __shfl_down_sync(FULL, u00.x, 1);
        if (lane == 0) w = (ok && x0 > 0) ? uc[row + x0 - 1] : 0.f;
        if (lane == 31) e = (ok && x0 + STRIP < nx) ? uc[row + x0 + STRIP] : 0.f;
        float4 v10 = zero4;
        if (ok) {
            float d[4], a[4];
            factors(r, src1, a1, d, a);
            v10 = fwd_row4(u00, w, e, u0m, u0p, p, c0, d, a);
        }
        const int rb = r - 1;
        const float w2 = __shfl_up_sync(FULL, v1m.w, 1), e2 = __shfl_down_sync(FULL, v1m.x, 1);
        if (own && rb >= y0 && rb < ny) {
            const int64_t rowb = (int64_t)rb * nx;
            float d[4], a[4];
            factors(rb, src2, a2, d, a);
            const float4 v2 = fwd_row4(v1m, w2, e2, v1m2, v10, u0m, cm, d, a);
            *reinterpret_cast<float4*>(u1 + rowb + i) = v1m;
            *reinterpret_cast<float4*>(u2 + rowb + i) = v2;
            if (ck1) *reinterpret_cast<float4*>(ck1 + rowb + i) = v1m;
            if (ck2) *reinterpret_cast<float4*>(ck2 + rowb + i) = v2;
        }
        u0m = u00; u00 = u0p;
        cm = c0;
        v1m2 = v1m; v1m = v10;
    }
}

template <int R>
void fwd2q_strip(const DevGeo& g, const float* coef, const Fwd2Step& s, cudaStream_t st) {
    const int rows_per_block = WARPS * R;
    dim3 grid((g.nx + 119) / 120, (g.ny + rows_per_block - 1) / rows_per_block + 1, s.ng);
    k_fwd2q_strip<R><<<grid, WARPS * 32, 0, st>>>(g, coef, s);
}

// Two forward steps per launch with the row inputs staged in shared memory (the forward
// counterpart of k_adj2s_strip): a per-warp ring of D rows of u(k) (row r+1), u(k-1) and the
// coefficient (row r), filled by 16-byte cp.async copies D rows ahead.  Strips start at
// x0 = 60 bx - 4 (16-byte aligned), lanes 1..30 write; the halo lanes' outer cells need no
// neighbour loads (no owned cell reads their first-step values).  Same arithmetic as
// k_fwd2_strip, so the results are identical.
constexpr int FS_ARR = 3;
constexpr int FS_ROW = FS_ARR * 64;

template <int R, int D>
__global__ void __launch_bounds__(WARPS * 32, 8) k_fwd2s_strip(DevGeo g, const float* __restrict__ coef, Fwd2Step s) {
    extern __shared__ float4 fs_mem4[];
    const int nx = g.nx, ny = g.ny;
    const int gl = blockIdx.z;
    if (blockIdx.y == gridDim.y - 1) {
        if (blockIdx.x != 0) return;
        if (s.gka >= 2) gather_slice(g, s.up + gl * s.gstride, gl, s.g0, s.gka, s.gmeas, s.gout);
        if (s.gkb >= 2) gather_slice(g, s.uc + gl * s.gstride, gl, s.g0, s.gkb, s.gmeas, s.gout);
        return;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x0 = blockIdx.x * 60 - 4;
    const int i = x0 + 2 * lane;
    const int y0 = (blockIdx.y * WARPS + warp) * R;
    if (y0 >= ny) return;
    float* ring = reinterpret_cast<float*>(fs_mem4) + warp * D * FS_ROW;
    const bool in = i >= 0 && i < nx;
    const bool own = in && lane >= 1 && lane <= 30;
    const float* uc = s.uc + gl * s.gstride;
    const float* up = s.up + gl * s.gstride;
    float* u1 = s.u1 + gl * s.gstride;
    float* u2 = s.u2 + gl * s.gstride;
    float* ck1 = s.ck1 ? s.ck1 + gl * s.ckstride : nullptr;
    float* ck2 = s.ck2 ? s.ck2 + gl * s.ckstride : nullptr;
    const bool edge_x = x0 < g.sponge_w || x0 + 64 > nx - g.sponge_w;
    const int32_t* em = g.emit + (int64_t)(s.g0 + gl) * g.gs;
    const bool src1 = s.k < g.n_src_steps, src2 = s.k + 1 < g.n_src_steps;
    const float a1 = src1 ? g.src[s.k] : 0.f, a2 = src2 ? g.src[s.k + 1] : 0.f;
    auto row_ok = [&](int r) { return in && r >= 0 && r < ny; };
    const int dca = edge_dist(i, nx), dcb = edge_dist(i + 1, nx);
    // copy duty: lanes 0-15 stage u(k) (row t+1) and the coefficient (row t), lanes 16-31
    // u(k-1) (row t); chunk (lane & 15) of each
    const int ch = lane & 15, half = lane >> 4;
    const int cx = x0 + 4 * ch;
    const bool cx_ok = cx >= 0 && cx + 3 < nx;
    const float* srcA = half ? up : uc;
    const unsigned ring_s = (unsigned)__cvta_generic_to_shared(ring) + 4u * (unsigned)(half * 64 + 4 * ch);
    auto stage = [&](int t, int slot) {
        const unsigned dst = ring_s + 4u * (unsigned)(slot * FS_ROW);
        const bool r1 = cx_ok && t + 1 >= 0 && t + 1 < ny, r0 = cx_ok && t >= 0 && t < ny;
        const int o0 = t * nx + cx;
        // slot layout: [0] u(k) row t+1, [1] u(k-1) row t, [2] coefficient row t
        if (half == 0) {
            cp_async16(dst, srcA + (r1 ? o0 + nx : 0), r1);
            cp_async16(dst + 4u * 2 * 64, coef + (r0 ? o0 : 0), r0);
        } else {
            cp_async16(dst, srcA + (r0 ? o0 : 0), r0);
        }
    };
    float2 u0m = ld2(uc, (y0 - 2) * nx + i, row_ok(y0 - 2));
    float2 u00 = ld2(uc, (y0 - 1) * nx + i, row_ok(y0 - 1));
    float2 cm = ld2(coef, (y0 - 2) * nx + i, row_ok(y0 - 2));
    float2 v1m2 = make_float2(0.f, 0.f), v1m = make_float2(0.f, 0.f);
    const int rlast = min(y0 + R, ny);
#pragma unroll
    for (int t = 0; t < D; ++t) {
        if (y0 - 1 + t <= rlast) stage(y0 - 1 + t, t);
        cp_async_commit();
    }
    int slot = 0;
#pragma unroll 1
    for (int r = y0 - 1; r <= rlast; ++r) {
        const int row = r * nx;
        const bool ok = row_ok(r);
        cp_async_wait<D - 1>();
        __syncwarp();
        const float* sr = ring + slot * FS_ROW + 2 * lane;
        const float2 u0p = *reinterpret_cast<const float2*>(sr);
        const float2 p = *reinterpret_cast<const float2*>(sr + 64);
        const float2 c0 = *reinterpret_cast<const float2*>(sr + 128);
        __syncwarp();
        if (r + D <= rlast) stage(r + D, slot);
        cp_async_commit();
        slot = slot + 1 == D ? 0 : slot + 1;
        // ---- u(k+1) at row r, all lanes (zero outside the grid)
        const float w = __shfl_up_sync(FULL, u00.y, 1), e = __shfl_down_sync(FULL, u00.x, 1);
        float2 v10 = make_float2(0.f, 0.f);
        if (ok) {
            const int dr = edge_dist(r, ny);
            const float drow = dr < g.sponge_w ? g.damp[dr] : 1.f;
            float dx = drow, dy = drow;
            if (edge_x) { dx = damp_at(g, dca, dr); dy = damp_at(g, dcb, dr); }
            const float ax = src1 ? emit_at(em, g.gs, row + i, a1) : 0.f;
            const float ay = src1 ? emit_at(em, g.gs, row + i + 1, a1) : 0.f;
            v10.x = fwd_cell(u00.y, w, u0m.x, u0p.x, u00.x, p.x, c0.x, dx, ax);
            v10.y = fwd_cell(e, u00.x, u0m.y, u0p.y, u00.y, p.y, c0.y, dy, ay);
        }
        // ---- u(k+2) at row r-1
        const int rb = r - 1;
        const float w2 = __shfl_up_sync(FULL, v1m.y, 1), e2 = __shfl_down_sync(FULL, v1m.x, 1);
        if (own && rb >= y0 && rb < ny) {
            const int rowb = rb * nx;
            const int dr = edge_dist(rb, ny);
            const float drow = dr < g.sponge_w ? g.damp[dr] : 1.f;
            float dx = drow, dy = drow;
            if (edge_x) { dx = damp_at(g, dca, dr); dy = damp_at(g, dcb, dr); }
            const float ax = src2 ? emit_at(em, g.gs, rowb + i, a2) : 0.f;
            const float ay = src2 ? emit_at(em, g.gs, rowb + i + 1, a2) : 0.f;
            float2 v2;
            v2.x = fwd_cell(v1m.y, w2, v1m2.x, v10.x, v1m.x, u0m.x, cm.x, dx, ax);
            v2.y = fwd_cell(e2, v1m.x, v1m2.y, v10.y, v1m.y, u0m.y, cm.y, dy, ay);
            *reinterpret_cast<float2*>(u1 + rowb + i) = v1m;
            *reinterpret_cast<float2*>(u2 + rowb + i) = v2;
            if (ck1) *reinterpret_cast<float2*>(ck1 + rowb + i) = v1m;
            if (ck2) *reinterpret_cast<float2*>(ck2 + rowb + i) = v2;
        }
        u0m = u00; u00 = u0p;
        cm = c0;
        v1m2 = v1m; v1m = v10;
    }
    cp_async_wait<0>();
}

template <int R, int D>
void fwd2s_strip(const DevGeo& g, const float* coef, const Fwd2Step& s, cudaStream_t st) {
    const int rows_per_block = WARPS * R;
    const size_t smem = sizeof(float) * WARPS * D * FS_ROW;
    dim3 grid((g.nx + 2 + 59) / 60, (g.ny + rows_per_block - 1) / rows_per_block + 1, s.ng);   // + gather row
    k_fwd2s_strip<R, D><<<grid, WARPS * 32, smem, st>>>(g, coef, s);
}

template <int R>
void fwd2_strip(const DevGeo& g, const float* coef, const Fwd2Step& s, cudaStream_t st) {
    const int rows_per_block = WARPS * R;
    dim3 grid((g.nx + 59) / 60, (g.ny + rows_per_block - 1) / rows_per_block + 1, s.ng);
    k_fwd2_strip<R><<<grid, WARPS * 32, 0, st>>>(g, coef, s);
}

// One forward step per launch with the row inputs staged in shared memory: a per-warp ring of
// D rows of u(k) (row j+1, with one 4-cell chunk of halo on each side), u(k-1) and the
// coefficient (row j), filled by 16-byte cp.async copies D rows ahead.  The west/east
// neighbours of every lane come from the staged halo row, so lanes 0 and 31 make no extra
// global loads.  Same arithmetic and sensor gather as k_fwd_strip: identical results.
constexpr int F1_UC = STRIP + 8;                 // u(k) row with halo: cells x0-4 .. x0+131
constexpr int F1_ROW = F1_UC + 2 * STRIP;        // + u(k-1) row + coefficient row

template <int R, int D>
__global__ void __launch_bounds__(WARPS * 32, 8) k_fwds_strip(DevGeo g, const float* __restrict__ coef, FwdStep s) {
    extern __shared__ float4 f1_mem4[];
    const int nx = g.nx, ny = g.ny;
    const int gl = blockIdx.z;
    if (blockIdx.y == gridDim.y - 1) {
        // sensor gather of slice k (k >= 2), one block per group
        if (blockIdx.x != 0 || s.gk < 2) return;
        const float* u = s.uc + gl * s.gstride;
        const int64_t base = ((int64_t)gl * g.nt + s.gk) * g.nch;
        const bool noisy = s.gmeas && g.noise_key;
        const uint64_t key = noisy ? *g.noise_key : 0;
        for (int c = threadIdx.x; c < g.nch; c += blockDim.x) {
            const int cell = g.rcv[c];
            float v = cell >= 0 ? u[cell] : 0.f;
            if (noisy) v *= noise_factor(key, g.noise_level, s.g0 + gl, s.gk, c);
            s.gout[base + c] = s.gmeas ? (cell >= 0 ? s.gmeas[base + c] - v : 0.f) : v;
        }
        return;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x0 = blockIdx.x * STRIP;
    const int i = x0 + 4 * lane;
    const int y0 = (blockIdx.y * WARPS + warp) * R;
    if (y0 >= ny) return;
    float* ring = reinterpret_cast<float*>(f1_mem4) + warp * D * F1_ROW;
    const bool act = i < nx;
    const float* uc = s.uc + gl * s.gstride;
    const float* up = s.up + gl * s.gstride;
    float* un = s.un + gl * s.gstride;
    float* ck = s.ck ? s.ck + gl * s.ckstride : nullptr;
    const bool edge_x = x0 < g.sponge_w || x0 + STRIP > nx - g.sponge_w;
    const bool src = s.k < g.n_src_steps;
    const int32_t* em = g.emit + (int64_t)(s.g0 + gl) * g.gs;
    const float a = src ? g.src[s.k] : 0.f;
    const int jend = min(y0 + R, ny);
    // copy duty: u(k) chunks lane (and 32 + lane for lanes 0, 1), u(k-1) and coefficient chunk lane
    const int cxu = x0 - 4 + 4 * lane, cxu2 = x0 + 124 + 4 * lane, cx = x0 + 4 * lane;
    const bool oku = cxu >= 0 && cxu + 3 < nx, oku2 = lane < 2 && cxu2 >= 0 && cxu2 + 3 < nx;
    const bool okc = cx + 3 < nx;
    const unsigned ring_s = (unsigned)__cvta_generic_to_shared(ring);
    auto stage = [&](int t, int slot) {              // row t: u(k) row t+1, u(k-1) and coefficient row t
        const unsigned dst = ring_s + 4u * (unsigned)(slot * F1_ROW);
        const bool r1 = t + 1 < ny, r0 = t < ny;     // t >= y0 >= 0
        const int o1 = (t + 1) * nx, o0 = t * nx;
        cp_async16(dst + 16u * lane, uc + (r1 && oku ? o1 + cxu : 0), r1 && oku);
        if (lane < 2) cp_async16(dst + 16u * (32 + lane), uc + (r1 && oku2 ? o1 + cxu2 : 0), r1 && oku2);
        cp_async16(dst + 4u * F1_UC + 16u * lane, up + (r0 && okc ? o0 + cx : 0), r0 && okc);
        cp_async16(dst + 4u * (F1_UC + STRIP) + 16u * lane, coef + (r0 && okc ? o0 + cx : 0), r0 && okc);
    };
    // rows y0-1 and y0 of u(k) and the neighbours of row y0 straight from global memory
    float4 rm = ld4(uc, (y0 - 1) * nx + i, act && y0 > 0);
    float4 r0 = ld4(uc, y0 * nx + i, act);
    float w0, e0;
    we(r0, uc + y0 * nx, lane, x0, nx, w0, e0);
#pragma unroll
    for (int t = 0; t < D; ++t) {
        if (y0 + t < jend) stage(y0 + t, t);
        cp_async_commit();
    }
    int slot = 0;
#pragma unroll 1
    for (int j = y0; j < jend; ++j) {
        const int row = j * nx;
        cp_async_wait<D - 1>();
        __syncwarp();
        const float* sr = ring + slot * F1_ROW;
        const float4 rp = *reinterpret_cast<const float4*>(sr + 4 + 4 * lane);
        const float wp = sr[3 + 4 * lane], ep = sr[8 + 4 * lane];     // neighbours of row j+1
        const float4 p = *reinterpret_cast<const float4*>(sr + F1_UC + 4 * lane);
        const float4 c = *reinterpret_cast<const float4*>(sr + F1_UC + STRIP + 4 * lane);
        __syncwarp();
        if (j + D < jend) stage(j + D, slot);
        cp_async_commit();
        slot = slot + 1 == D ? 0 : slot + 1;
        const bool near = edge_x || j < g.sponge_w || j >= ny - g.sponge_w;
        const float dx = near ? sponge(g, i, j) : 1.f;
        const float dy = near ? sponge(g, i + 1, j) : 1.f;
        const float dz = near ? sponge(g, i + 2, j) : 1.f;
        const float dw = near ? sponge(g, i + 3, j) : 1.f;
        const int64_t q0 = row + i;
        const float ax = src ? emit_at(em, g.gs, q0, a) : 0.f;
        const float ay = src ? emit_at(em, g.gs, q0 + 1, a) : 0.f;
        const float az = src ? emit_at(em, g.gs, q0 + 2, a) : 0.f;
        const float aw = src ? emit_at(em, g.gs, q0 + 3, a) : 0.f;
        float4 v;
        v.x = fwd_cell(r0.y, w0, rm.x, rp.x, r0.x, p.x, c.x, dx, ax);
        v.y = fwd_cell(r0.z, r0.x, rm.y, rp.y, r0.y, p.y, c.y, dy, ay);
        v.z = fwd_cell(r0.w, r0.y, rm.z, rp.z, r0.z, p.z, c.z, dz, az);
        v.w = fwd_cell(e0, r0.z, rm.w, rp.w, r0.w, p.w, c.w, dw, aw);
        if (act) {
            *reinterpret_cast<float4*>(un + row + i) = v;
            if (ck) *reinterpret_cast<float4*>(ck + row + i) = v;
        }
        rm = r0; r0 = rp; w0 = wp; e0 = ep;
    }
    cp_async_wait<0>();
}

// ---------------------------------------------------------------------------
// One forward step, lean form: four cells per lane (128-cell strips), R rows per warp in a fully
// unrolled loop with every access predicated instead of branched, the sponge factor from the
// per-cell map (one 128-bit load per row instead of per-cell edge-distance lookups), the source
// term only in launches of source steps (SRC), the west / east neighbours of a lane's four cells
// by shuffles with one predicated scalar load at each strip end.  Same cell arithmetic
// (fwd_cell) as every other forward kernel, so the same bits.
template <int R, bool SRC, bool PF>
__global__ void __launch_bounds__(WARPS * 32, PF ? 7 : 8) k_fwdl_strip(DevGeo g, const float* __restrict__ coef, FwdStep s) {
    const int nx = g.nx, ny = g.ny;
    const int gl = blockIdx.z;
    if (blockIdx.y == gridDim.y - 1) {
        // sensor gather of slice k (k >= 2), one block per group
        if (blockIdx.x != 0 || s.gk < 2) return;
        const float* u = s.uc + gl * s.gstride;
        const int64_t base = ((int64_t)gl * g.nt + s.gk) * g.nch;
        const bool noisy = s.gmeas && g.noise_key;
        const uint64_t key = noisy ? *g.noise_key : 0;
        for (int c = threadIdx.x; c < g.nch; c += blockDim.x) {
            const int cell = g.rcv[c];
            float v = cell >= 0 ? u[cell] : 0.f;
            if (noisy) v *= noise_factor(key, g.noise_level, s.g0 + gl, s.gk, c);
            s.gout[base + c] = s.gmeas ? (cell >= 0 ? s.gmeas[base + c] - v : 0.f) : v;
        }
        return;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x0 = blockIdx.x * STRIP;
    const int i = x0 + 4 * lane;
    const int y0 = (blockIdx.y * WARPS + warp) * R;
    if (y0 >= ny) return;
    const bool act = i < nx;                         // nx % 4 == 0: a lane's four cells are all in or out
    const float* __restrict__ uc = s.uc + gl * s.gstride;
    const float* __restrict__ up = s.up + gl * s.gstride;
    float* __restrict__ un = s.un + gl * s.gstride;
    float* __restrict__ ck = s.ck ? s.ck + gl * s.ckstride : nullptr;
    const float* __restrict__ dmap = g.dmap;
    // lane 0 reads the cell west of the strip, lane 31 the cell east of it
    const int xs = lane == 0 ? x0 - 1 : x0 + STRIP;
    const bool side = (lane == 0 && x0 > 0) || (lane == 31 && x0 + STRIP < nx);
    const int ggl = s.g0 + gl;
    const float a = SRC ? g.src[s.k] : 0.f;
    int o = y0 * nx;                                  // row offset (32-bit: the strip path needs nx*ny < 2^31)
    float4 rm = ld4(uc, o - nx + i, act && y0 > 0);
    float4 r0 = ld4(uc, o + i, act);
    float sc0 = side ? uc[o + xs] : 0.f;
    // PF: the inputs of row r+1 are requested before row r is computed (two rows of loads in flight)
    float4 q_rp, q_p, q_c, q_d;
    float q_sc = 0.f;
    if (PF) {
        q_rp = ld4(uc, o + nx + i, act && y0 + 1 < ny);
        q_sc = side && y0 + 1 < ny ? uc[o + nx + xs] : 0.f;
        q_p = ld4(up, o + i, act);
        q_c = ld4(coef, o + i, act);
        q_d = ld4(dmap, o + i, act);
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int j = y0 + r;
        const bool okj = act && j < ny;
        float4 rp, p, c, d;
        float scp;
        if (PF) {
            rp = q_rp; p = q_p; c = q_c; d = q_d; scp = q_sc;
            if (r + 1 < R) {
                const bool ok1 = act && j + 1 < ny, ok2 = act && j + 2 < ny;
                q_rp = ld4(uc, o + 2 * nx + i, ok2);
                q_sc = side && j + 2 < ny ? uc[o + 2 * nx + xs] : 0.f;
                q_p = ld4(up, o + nx + i, ok1);
                q_c = ld4(coef, o + nx + i, ok1);
                q_d = ld4(dmap, o + nx + i, ok1);
            }
        } else {
            const bool okn = act && j + 1 < ny;
            rp = ld4(uc, o + nx + i, okn);
            scp = side && j + 1 < ny ? uc[o + nx + xs] : 0.f;
            p = ld4(up, o + i, okj);
            c = ld4(coef, o + i, okj);
            d = ld4(dmap, o + i, okj);
        }
        float w = __shfl_up_sync(FULL, r0.w, 1), e = __shfl_down_sync(FULL, r0.x, 1);
        if (lane == 0) w = sc0;
        if (lane == 31) e = sc0;
        float ax = 0.f, ay = 0.f, az = 0.f, aw = 0.f;
        if (SRC && okj) {
            const int4 rid = *reinterpret_cast<const int4*>(g.rid + o + i);
            ax = rid.x >= 0 && rid.x / g.gs == ggl ? a : 0.f;
            ay = rid.y >= 0 && rid.y / g.gs == ggl ? a : 0.f;
            az = rid.z >= 0 && rid.z / g.gs == ggl ? a : 0.f;
            aw = rid.w >= 0 && rid.w / g.gs == ggl ? a : 0.f;
        }
        float4 v;
        v.x = fwd_cell(r0.y, w, rm.x, rp.x, r0.x, p.x, c.x, d.x, ax);
        v.y = fwd_cell(r0.z, r0.x, rm.y, rp.y, r0.y, p.y, c.y, d.y, ay);
        v.z = fwd_cell(r0.w, r0.y, rm.z, rp.z, r0.z, p.z, c.z, d.z, az);
        v.w = fwd_cell(e, r0.z, rm.w, rp.w, r0.w, p.w, c.w, d.w, aw);
        if (okj) {
            *reinterpret_cast<float4*>(un + o + i) = v;
            if (ck) *reinterpret_cast<float4*>(ck + o + i) = v;
        }
        rm = r0;
        r0 = rp;
        sc0 = scp;
        o += nx;
    }
}

template <int R, bool PF = false>
void fwdl_strip(const DevGeo& g, const float* coef, const FwdStep& s, cudaStream_t st) {
    const int rows_per_block = WARPS * R;
    dim3 grid((g.nx + STRIP - 1) / STRIP, (g.ny + rows_per_block - 1) / rows_per_block + 1, s.ng);
    if (s.k < g.n_src_steps) k_fwdl_strip<R, true, PF><<<grid, WARPS * 32, 0, st>>>(g, coef, s);
    else k_fwdl_strip<R, false, PF><<<grid, WARPS * 32, 0, st>>>(g, coef, s);
}

template <int R, int D>
void fwds_strip(const DevGeo& g, const float* coef, const FwdStep& s, cudaStream_t st) {
    const int rows_per_block = WARPS * R;
    const size_t smem = sizeof(float) * WARPS * D * F1_ROW;
    dim3 grid((g.nx + STRIP - 1) / STRIP, (g.ny + rows_per_block - 1) / rows_per_block + 1, s.ng);
    k_fwds_strip<R, D><<<grid, WARPS * 32, smem, st>>>(g, coef, s);
}

template <int R>
void fwd_strip(const DevGeo& g, const float* coef, const FwdStep& s, cudaStream_t st) {
    const int rows_per_block = WARPS * R;
    dim3 grid((g.nx + STRIP - 1) / STRIP, (g.ny + rows_per_block - 1) / rows_per_block + 1, s.ng);
    k_fwd_strip<R><<<grid, WARPS * 32, 0, st>>>(g, coef, s);
}

template <int R>
void adj_strip(int variant, const DevGeo& g, const float* coef, const AdjStep& s, cudaStream_t st) {
    const int rows_per_block = WARPS * R;
    dim3 grid((g.nx + STRIP - 1) / STRIP, (g.ny + rows_per_block - 1) / rows_per_block, s.ng);
    switch (variant) {
    case 1: k_adj_strip<R, 8, 1><<<grid, WARPS * 32, 0, st>>>(g, coef, s); break;
    case 2: k_adj_strip<R, 1, 1><<<grid, WARPS * 32, 0, st>>>(g, coef, s); break;
    case 3: k_adj_strip<R, 6, 2><<<grid, WARPS * 32, 0, st>>>(g, coef, s); break;
    default: k_adj_strip<R, 1, 2><<<grid, WARPS * 32, 0, st>>>(g, coef, s); break;
    }
}

}  // namespace

void launch_resid_parts(const float* rr, int ng, int nt, int nch, double* part, void* stream) {
    k_resid_parts<<<dim3(nt, ng), 256, 0, (cudaStream_t)stream>>>(rr, nt, nch, part);
}

// The strip kernels index a slice with 32-bit offsets.
bool strip_supported(const DevGeo& g, int profile) {
    return profile == TOMO_PROFILE_CFG && g.nx % 4 == 0 && (int64_t)g.nx * (g.ny + 2) < ((int64_t)1 << 31) &&
           g.rbits != nullptr;
}

void launch_fwd2_strip(int rows, const DevGeo& g, const float* coef, const FwdStep& a, const FwdStep& b,
                       bool gather_prev, bool gather_cur, void* stream) {
    Fwd2Step s{};
    s.up = a.up; s.uc = a.uc; s.u1 = a.un; s.u2 = b.un; s.gstride = a.gstride;
    s.ck1 = a.ck; s.ck2 = b.ck; s.ckstride = a.ck ? a.ckstride : b.ckstride;
    s.k = a.k; s.g0 = a.g0; s.ng = a.ng;
    s.gmeas = a.gmeas; s.gout = a.gout;
    s.gka = (a.gout && gather_prev) ? a.k - 1 : -1;   // slice k-1, read from a.up
    s.gkb = (a.gout && gather_cur) ? a.k : -1;        // slice k, read from a.uc
    cudaStream_t st = (cudaStream_t)stream;
    switch (rows) {
    case 4: fwd2_strip<4>(g, coef, s, st); break;
    case 16: fwd2_strip<16>(g, coef, s, st); break;
    case 32: fwd2_strip<32>(g, coef, s, st); break;
    case 104: fwd2q_strip<4>(g, coef, s, st); break;
    case 108: fwd2q_strip<8>(g, coef, s, st); break;
    case 116: fwd2q_strip<16>(g, coef, s, st); break;
    case 132: fwd2q_strip<32>(g, coef, s, st); break;
    case 3204: fwd2s_strip<4, 2>(g, coef, s, st); break;     // 3000 + 100 D + rows: staged
    case 3208: fwd2s_strip<8, 2>(g, coef, s, st); break;
    case 3216: fwd2s_strip<16, 2>(g, coef, s, st); break;
    case 3232: fwd2s_strip<32, 2>(g, coef, s, st); break;
    case 3304: fwd2s_strip<4, 3>(g, coef, s, st); break;
    case 3308: fwd2s_strip<8, 3>(g, coef, s, st); break;
    case 3316: fwd2s_strip<16, 3>(g, coef, s, st); break;
    case 3332: fwd2s_strip<32, 3>(g, coef, s, st); break;
    default: fwd2_strip<8>(g, coef, s, st); break;
    }
}

void launch_adj2_strip(int rows, const DevGeo& g, const float* coef, const AdjStep& a, const AdjStep& b,
                       void* stream) {
    Adj2Step s{};
    s.z2 = a.z2; s.z1 = a.z1; s.za = a.zk; s.zb = b.zk; s.zstride = a.zstride;
    s.ua = a.uq; s.ub = b.uq; s.ustride = a.ustride;
    s.rra = a.rr; s.rrb = b.rr; s.rrstride = a.rrstride;
    s.corr = a.corr; s.cstride = a.cstride; s.ng = a.ng;
    cudaStream_t st = (cudaStream_t)stream;
    // code = rows + 100 * AHEAD + 1000 * SPLIT (see k_adj2_strip); 2000 + rows: k_adj2q_strip
#define ADJ2_CASE(R, A, S) \
    case (R) + 100 * (A) + 1000 * (S): adj2_strip<R, A, S>(g, coef, s, st); return;
#define ADJ2_ROWS(A, S) ADJ2_CASE(4, A, S) ADJ2_CASE(8, A, S) ADJ2_CASE(16, A, S) ADJ2_CASE(32, A, S)
    switch (rows) {
        ADJ2_ROWS(0, false) ADJ2_ROWS(1, false) ADJ2_ROWS(2, false)
        ADJ2_ROWS(0, true) ADJ2_ROWS(1, true) ADJ2_ROWS(2, true)
    case 4004: adj2_strip<4, 0, false, true>(g, coef, s, st); return;     // 4000 + rows + 100 AHEAD: PACK
    case 4008: adj2_strip<8, 0, false, true>(g, coef, s, st); return;
    case 4016: adj2_strip<16, 0, false, true>(g, coef, s, st); return;
    case 4032: adj2_strip<32, 0, false, true>(g, coef, s, st); return;
    case 4104: adj2_strip<4, 1, false, true>(g, coef, s, st); return;
    case 4108: adj2_strip<8, 1, false, true>(g, coef, s, st); return;
    case 4116: adj2_strip<16, 1, false, true>(g, coef, s, st); return;
    case 4132: adj2_strip<32, 1, false, true>(g, coef, s, st); return;
    case 3204: adj2s_strip<4, 2>(g, coef, s, st); return;    // 3000 + 100 D + rows: staged, D rows ahead
    case 3208: adj2s_strip<8, 2>(g, coef, s, st); return;
    case 3216: adj2s_strip<16, 2>(g, coef, s, st); return;
    case 3232: adj2s_strip<32, 2>(g, coef, s, st); return;
    case 3304: adj2s_strip<4, 3>(g, coef, s, st); return;
    case 3308: adj2s_strip<8, 3>(g, coef, s, st); return;
    case 3316: adj2s_strip<16, 3>(g, coef, s, st); return;
    case 3332: adj2s_strip<32, 3>(g, coef, s, st); return;
    case 3404: adj2s_strip<4, 4>(g, coef, s, st); return;
    case 3408: adj2s_strip<8, 4>(g, coef, s, st); return;
    case 3416: adj2s_strip<16, 4>(g, coef, s, st); return;
    case 3432: adj2s_strip<32, 4>(g, coef, s, st); return;
    case 9208: adj2s4_strip<8, 2, 4>(g, coef, s, st); return;   // 9000 + 100 D + rows: staged, 4 cells/lane
    case 9308: adj2s4_strip<8, 3, 4>(g, coef, s, st); return;
    case 9216: adj2s4_strip<16, 2, 3>(g, coef, s, st); return;
    case 9316: adj2s4_strip<16, 3, 3>(g, coef, s, st); return;
    case 8208: adj2s_strip<8, 2, 6, true>(g, coef, s, st); return;    // 8000 + 100 D + rows: staged, unrolled
    case 8308: adj2s_strip<8, 3, 6, true>(g, coef, s, st); return;
    case 8408: adj2s_strip<8, 4, 6, true>(g, coef, s, st); return;
    case 8316: adj2s_strip<16, 3, 6, true>(g, coef, s, st); return;
    case 18208: adj2s_strip<8, 2, 5, true, true>(g, coef, s, st); return;   // 10000 + unrolled staged: packed FP32x2, 5 blocks
    case 18308: adj2s_strip<8, 3, 5, true, true>(g, coef, s, st); return;
    case 18408: adj2s_strip<8, 4, 5, true, true>(g, coef, s, st); return;
    case 5216: adj2s_strip<16, 2, 8>(g, coef, s, st); return;   // 5000 + 100 D + rows: staged, 8 blocks
    case 5232: adj2s_strip<32, 2, 8>(g, coef, s, st); return;
    case 5316: adj2s_strip<16, 3, 8>(g, coef, s, st); return;
    case 5332: adj2s_strip<32, 3, 8>(g, coef, s, st); return;
    case 7008: adjl2_strip<8, 4>(g, coef, s, st); return;   // 7000 + rows (+ 100: 3 blocks): lean
    case 7016: adjl2_strip<16, 4>(g, coef, s, st); return;
    case 7108: adjl2_strip<8, 3>(g, coef, s, st); return;
    case 7116: adjl2_strip<16, 3>(g, coef, s, st); return;
    case 2004: adj2q_strip<4>(g, coef, s, st); return;     // 2000 + rows: four cells per lane
    case 2008: adj2q_strip<8>(g, coef, s, st); return;
    case 2016: adj2q_strip<16>(g, coef, s, st); return;
    case 2032: adj2q_strip<32>(g, coef, s, st); return;
    default: adj2_strip<8, 0, false>(g, coef, s, st); return;
    }
#undef ADJ2_ROWS
#undef ADJ2_CASE
}

void launch_fwd_strip(int rows, const DevGeo& g, const float* coef, const FwdStep& s, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    switch (rows) {   // 3000 + 100 D + rows: inputs staged in shared memory D rows ahead; 6000 + rows: lean
    case 6004: fwdl_strip<4>(g, coef, s, st); break;
    case 6008: fwdl_strip<8>(g, coef, s, st); break;
    case 6016: fwdl_strip<16>(g, coef, s, st); break;
    case 6104: fwdl_strip<4, true>(g, coef, s, st); break;   // 6100 + rows: lean, next row requested ahead
    case 6108: fwdl_strip<8, true>(g, coef, s, st); break;
    case 6116: fwdl_strip<16, true>(g, coef, s, st); break;
    case 3204: fwds_strip<4, 2>(g, coef, s, st); break;
    case 3208: fwds_strip<8, 2>(g, coef, s, st); break;
    case 3216: fwds_strip<16, 2>(g, coef, s, st); break;
    case 3304: fwds_strip<4, 3>(g, coef, s, st); break;
    case 3308: fwds_strip<8, 3>(g, coef, s, st); break;
    case 3316: fwds_strip<16, 3>(g, coef, s, st); break;
    case 2: fwd_strip<2>(g, coef, s, st); break;
    case 4: fwd_strip<4>(g, coef, s, st); break;
    case 16: fwd_strip<16>(g, coef, s, st); break;
    case 32: fwd_strip<32>(g, coef, s, st); break;
    default: fwd_strip<8>(g, coef, s, st); break;
    }
}

void launch_adj_strip(int rows, int variant, const DevGeo& g, const float* coef, const AdjStep& s, void* stream) {
    cudaStream_t st = (cudaStream_t)stream;
    switch (rows) {
    case 2: adj_strip<2>(variant, g, coef, s, st); break;
    case 4: adj_strip<4>(variant, g, coef, s, st); break;
    case 16: adj_strip<16>(variant, g, coef, s, st); break;
    case 32: adj_strip<32>(variant, g, coef, s, st); break;
    default: adj_strip<8>(variant, g, coef, s, st); break;
    }
}

}  // namespace tomo
