// cell.cuh -- per-cell arithmetic and small helpers shared by the warp-strip kernels
// (strip.cu) and the multi-step tile kernels (tile.cu) of the benchmark-profile physics.
//
// Every kernel that advances a cell evaluates it with the helpers below, in the same
// operation order, so the kernels give identical bits whatever their structure (strips of one
// or two steps per launch, tiles of several steps per launch).  Included inside
// namespace tomo { namespace { ... } } of each translation unit.
#pragma once
constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ float4 ld4(const float* __restrict__ p, int64_t off, bool ok) {
    return ok ? *reinterpret_cast<const float4*>(p + off) : make_float4(0.f, 0.f, 0.f, 0.f);
}

// Sponge factor of cell (i, j): a table lookup by the distance to the nearest edge.
__device__ __forceinline__ float sponge(const DevGeo& g, int i, int j) {
    const int dd = min(min(i, j), min(g.nx - 1 - i, g.ny - 1 - j));
    return dd < g.sponge_w ? g.damp[dd] : 1.f;
}

// Cell arithmetic with explicit rounding (products, sums and fused multiply-adds as written):
// every kernel evaluates cells with these, so their results agree bit for bit whatever the
// compiler would otherwise contract.
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }

// Packed FP32x2 arithmetic (add/sub/mul/fma .rn.f32x2, sm_100 and later): one instruction for
// a lane's two cells, each half rounded exactly as the scalar __fadd_rn / __fsub_rn /
// __fmul_rn / __fmaf_rn, so results match the one-cell helpers bit for bit.
__device__ __forceinline__ float2 pk_add(float2 a, float2 b) {
    float2 r;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "add.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ float2 pk_sub(float2 a, float2 b) {
    float2 r;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ float2 pk_mul(float2 a, float2 b) {
    float2 r;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "mul.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ float2 pk_fma(float2 a, float2 b, float2 c) {
    float2 r;
    asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "mov.b64 rc, {%6, %7};\n\tfma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(r.x), "=f"(r.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return r;
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return make_float2(mul(a.x, b.x), mul(a.y, b.y)); }
__device__ __forceinline__ float4 mul4(float4 a, float4 b) {
    return make_float4(mul(a.x, b.x), mul(a.y, b.y), mul(a.z, b.z), mul(a.w, b.w));
}

// d * ((2 z - z2) + ((((ce + cw) + cs) + cn) - 4 cz) + inj), where cz = c z and the
// neighbour products c z are passed in rounded.  2 z and 4 cz are exact (power-of-two scales),
// so the fused forms round exactly as a multiply followed by an add would.
__device__ __forceinline__ float adj_cell(float ce, float cw, float cs, float cn, float cz, float z, float z2,
                                          float inj, float d) {
    const float lz = __fmaf_rn(-4.f, cz, __fadd_rn(__fadd_rn(__fadd_rn(ce, cw), cs), cn));
    return mul(d, __fadd_rn(__fadd_rn(__fmaf_rn(2.f, z, -z2), lz), inj));
}

// ((e + w) + s) + n - 4 u
__device__ __forceinline__ float lap5(float e, float w, float s, float n, float u) {
    return __fmaf_rn(-4.f, u, __fadd_rn(__fadd_rn(__fadd_rn(e, w), s), n));
}

// adj_cell and lap5 for a lane's two cells in packed FP32x2 (same operation order and rounding)
__device__ __forceinline__ float2 adj_cell2(float2 ce, float2 cw, float2 cs, float2 cn, float2 cz, float2 z, float2 z2,
                                            float2 inj, float2 d) {
    const float2 lz = pk_fma(make_float2(-4.f, -4.f), cz, pk_add(pk_add(pk_add(ce, cw), cs), cn));
    return pk_mul(d, pk_add(pk_add(pk_sub(pk_mul(make_float2(2.f, 2.f), z), z2), lz), inj));
}
__device__ __forceinline__ float2 lap5_2(float2 e, float2 w, float2 s, float2 n, float2 u) {
    return pk_fma(make_float2(-4.f, -4.f), u, pk_add(pk_add(pk_add(e, w), s), n));
}

// Forward cell update d ((2 u - up) + c lap) + a with fused multiply-adds (shared by every
// forward kernel): (2 u - up) is rounded once, then c lap + that, then d times that plus a.
__device__ __forceinline__ float fwd_cell(float e, float w, float s, float n, float u, float up, float c, float d,
                                          float a) {
    return __fmaf_rn(d, __fmaf_rn(c, lap5(e, w, s, n, u), __fmaf_rn(2.f, u, -up)), a);
}

// Source amplitude a at cell q of group g at step k (0 when q emits nothing).
__device__ __forceinline__ float emit_at(const int32_t* em, int gs, int64_t q, float a) {
    float r = 0.f;
    for (int t = 0; t < gs; ++t)
        if (em[t] == q) r += a;
    return r;
}

// Receiver bitmap (g.rbits: per row, one bit per 32-cell block, g.rwords words per row) words
// and masks covering a strip's cells [xa, xb); a strip of at most 128 cells spans at most two
// words.  Strips whose rows have no receiver never read the per-cell receiver map.
struct RcvMask {
    int w0, w1;
    uint32_t m0, m1;
};

__device__ __forceinline__ RcvMask rcv_mask(const DevGeo& g, int xa, int xb) {
    xa = max(xa, 0);
    xb = min(xb, g.nx);
    RcvMask k{0, 0, 0u, 0u};
    if (xa >= xb) return k;
    const int b0 = xa >> 5, b1 = (xb - 1) >> 5;
    k.w0 = b0 >> 5;
    k.w1 = b1 >> 5;
    const uint32_t lo = ~0u << (b0 & 31);
    const uint32_t hi = (b1 & 31) == 31 ? ~0u : ((1u << ((b1 & 31) + 1)) - 1u);
    if (k.w0 == k.w1) {
        k.m0 = lo & hi;
    } else {
        k.m0 = lo;
        k.m1 = hi;
    }
    return k;
}

// Whether row r has a receiver in the strip (the same answer for the whole warp).
__device__ __forceinline__ bool rcv_row(const DevGeo& g, const RcvMask& k, int r) {
    if (r < 0 || r >= g.ny) return false;
    const uint32_t* w = g.rbits + (int64_t)r * g.rwords;
    return ((w[k.w0] & k.m0) | (k.m1 ? (w[k.w1] & k.m1) : 0u)) != 0u;
}

// Distance of index i to the nearer end of [0, n), clamped at 0 for indices outside.
__device__ __forceinline__ int edge_dist(int i, int n) { return max(0, min(i, n - 1 - i)); }

// Sponge factor from a cell's column and row edge distances (equal to sponge(g, i, j)).
__device__ __forceinline__ float damp_at(const DevGeo& g, int dcol, int drow) {
    const int dd = min(dcol, drow);
    return dd < g.sponge_w ? g.damp[dd] : 1.f;
}

// 16-byte asynchronous global-to-shared copy (cp.async, L2 only); ok == false zero-fills the
// destination without reading the source.
__device__ __forceinline__ void cp_async16(unsigned smem_addr, const float* gmem, bool ok) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_addr), "l"(gmem), "r"(ok ? 16 : 0));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// Programmatic dependent launch: a kernel launched by launch_pdl may start while the kernel
// before it in the stream finishes.  Such a kernel reads nothing another kernel writes before
// grid_dep_wait() (which returns once the previous kernel has completed and its writes are
// visible; at once for a plain launch), then lets the next launch start early.
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void grid_dep_trigger() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

// Launch that may overlap the end of the previous kernel in the stream (programmatic stream
// serialization); TOMO_NO_PDL=1 launches in plain stream order.
template <typename Kern, typename... Args>
void launch_pdl(Kern kern, dim3 grid, int tpb, size_t smem, void* stream, const Args&... args) {
    static const bool off = [] {
        const char* e = std::getenv("TOMO_NO_PDL");
        return e && *e && *e != '0';
    }();
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(tpb);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = (cudaStream_t)stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = off ? 0 : 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kern, args...);
    if (e != cudaSuccess && std::getenv("TOMO_DEBUG_LAUNCH")) {
        cudaFuncAttributes fa{};
        cudaFuncGetAttributes(&fa, kern);
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        cudaStreamIsCapturing((cudaStream_t)stream, &cs);
        std::fprintf(stderr, "tomo: launch (grid %u x %u, %d threads, %zu B shared; max dynamic %d, static %zu, "
                     "regs %d, max threads %d, capturing %d) failed: %s\n", grid.x, grid.y, tpb, smem,
                     fa.maxDynamicSharedSizeBytes, fa.sharedSizeBytes, fa.numRegs, fa.maxThreadsPerBlock, (int)cs,
                     cudaGetErrorString(e));
    }
}


// Cooperative launch: every block is resident at once (the kernel's blocks wait on one another
// at grid barriers), in stream order after the previous kernel.
template <typename Kern, typename... Args>
void launch_coop(Kern kern, dim3 grid, int tpb, size_t smem, void* stream, const Args&... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(tpb);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = (cudaStream_t)stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kern, args...);
    if (e != cudaSuccess && std::getenv("TOMO_DEBUG_LAUNCH"))
        std::fprintf(stderr, "tomo: cooperative launch (grid %u x %u, %d threads, %zu B shared) failed: %s\n", grid.x,
                     grid.y, tpb, smem, cudaGetErrorString(e));
}

