// Host driver of the Static3D GPU solver and its C ABI (include/plgpu_fem3d.h).
//
// The handle mirrors the state PLaSK's ThermalFem3DSolver keeps between calls
// (solvers/thermal/static/therm3d.hpp:31-39): the temperature field persists on
// the device across compute() calls and is reset by invalidate().  Boundary
// conditions are materialised once per change into compact device lists; the
// volume operator is applied matrix-free from per-element conductivities.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/plgpu_elec3d.h"
#include "../../include/plgpu_fem2d.h"
#include "../../include/plgpu_fem3d.h"
#include "../../include/plgpu_unet.h"
#include "elec3d_kernels.h"
#include "fem2d_kernels.h"
#include "fem3d_device.cuh"
#include "fem3d_kernels.h"
#include "unet.h"

#include <nvtx3/nvToolsExt.h>

using namespace plgpu;

namespace {

constexpr double kSB = 5.670373e-8;  // plask/phys/constants.hpp:41
constexpr int kMaxOuterLoops = 100000;

struct CudaError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct ArgError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct StateError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct SolveError : std::runtime_error {
    int code;
    SolveError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

// NVTX range for the phases of a computation (outer loop, setMatrix, linear solve, time
// step): visible on a profiler's timeline, a no-op when no tool is attached.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// RAII device allocation
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    void alloc(size_t nbytes) {
        if (nbytes == bytes && p) return;
        release();
        if (nbytes == 0) return;
        ck(cudaMalloc(&p, nbytes), "cudaMalloc");
        bytes = nbytes;
    }
    template <typename T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

template <typename T>
void upload(DevBuf& d, const std::vector<T>& v, cudaStream_t s) {
    d.alloc(v.size() * sizeof(T));
    if (!v.empty()) ck(cudaMemcpyAsync(d.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s), "upload");
}

}  // namespace

// ---------------------------------------------------------------------------------------
// Multiply without allocation (plgpu_fem3d_mult_noalloc).
//
// Some callers cannot allocate device memory at the moment they need A x: a host
// framework that has reserved the whole GPU for its own caching allocator (cudaMalloc
// fails), or a latency-critical loop on other streams that cannot afford the
// device-wide synchronisation cudaMalloc and cudaFree may cause.  plgpu_fem3d_mult stages the vectors in a
// buffer it allocates per call; plgpu_fem3d_mult_noalloc stages them in the
// file-scope array below instead (16 MiB).
//
// Host code cannot use the array's name as a device address (in host code it names a
// host-side shadow), so its address is looked up with cudaGetSymbolAddress, once per
// device, when a handle is set up on that device (noalloc_setup, called from
// setup_mesh).  Looking it up loads this file's module onto the device, which under
// CUDA's lazy module loading is when the driver allocates the array; doing it at set-up,
// where the handle allocates its own buffers anyway, keeps that allocation out of the
// call.  From then on the device holds the array until the process exits.
//
// The array is shared by all calls and all handles and keeps the last call's
// contents.  Nothing in it needs to start at zero: every word a call reads is
// written by the same call first.  Calls that overlap on the GPU (two handles on
// two streams at the same time) race on it.

namespace {
constexpr size_t kNoAllocMaxNodes = size_t(1) << 21;  // 2,097,152 nodes
constexpr int kNoAllocMaxDevices = 64;
__device__ __align__(256) double g_noalloc_stage[kNoAllocMaxNodes];

std::mutex g_noalloc_mutex;
double* g_noalloc_ptr[kNoAllocMaxDevices] = {};  // device address of g_noalloc_stage, per device

// Look up the staging array's device address on device `dev` (the current device) once.
void noalloc_setup(int dev) {
    if (dev < 0 || dev >= kNoAllocMaxDevices) return;  // mult_noalloc rejects such devices
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        ck(cudaGetSymbolAddress(&p, g_noalloc_stage), "cudaGetSymbolAddress");
        g_noalloc_ptr[dev] = static_cast<double*>(p);
    }
}

// The address looked up at set-up for device `dev`, or nullptr.
double* noalloc_stage(int dev) {
    if (dev < 0 || dev >= kNoAllocMaxDevices) return nullptr;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    return g_noalloc_ptr[dev];
}
}  // namespace

struct plgpu_unet {
    std::string err;
    UNetModel model;
};

struct plgpu_fem3d {
    std::string err;
    // mesh
    int n[3] = {0, 0, 0};
    long long N = 0, NE = 0;
    int ordering = PLGPU_ORDER_012;
    int major = 0, medium = 1, minor = 2;
    long long ns[3] = {0, 0, 0};  // mesh-order node strides of axes 0/1/2
    long long es[3] = {0, 0, 0};  // mesh-order element strides
    std::vector<double> ax[3];
    // 0: 3D; PLGPU_GEOMETRY_CARTESIAN / _CYLINDRICAL: a 2D mesh (axes 0 and 1) stored as
    // one node plane, n[2] = 1, whose elements are the quads of axes 0 and 1
    int planar = 0;
    DevBuf rmid64, rmid32;  // cylindrical: midpoint radius of every element column
    cudaStream_t stream = nullptr;
    int device = 0;  // the device current at set-up, which owns the stream and every buffer
    LaunchCfg cfg{};
    int sm_count = 0;

    DevBuf h64[3], r64[3], h32[3], r32[3], z64;
    DevBuf zf64, zr64, zf32, zr32;  // dz / 48 and 1 / (48 dz) per element layer
    GridT<double> g64{};
    GridT<float> g32{};

    // materials
    int n_mat = 0;
    std::vector<double> k300, pexp, kzr, hexp;
    std::vector<uint8_t> empty;
    bool aniso = false;
    DevBuf d_k300, d_p, d_kzr, d_hexp, d_excl;
    MatTable tab{};
    // tabulated k(T) per material (empty: the power law)
    std::vector<std::vector<double>> ktab_T, ktab_xy, ktab_z;
    DevBuf d_toff, d_tn, d_tT, d_txy, d_tz;
    bool any_ktab = false;

    // elements (canonical padded layout)
    std::vector<int32_t> host_mat;  // mesh element order
    DevBuf d_mat, d_heat, d_th, d_hleaf;
    bool have_elements = false, have_leaf = false, heat_dirty = true;

    // fields
    DevBuf T, T0, F, b, r64v, vD, diag, minv64, minv32, k64, k32, kz64, kz32;
    DevBuf p64, q64, x32, r32v, p32, q32;
    DevBuf partials, d_ctl;
    SolveCtl* h_ctl = nullptr;

    // boundary conditions as appended
    struct Cond {
        std::vector<int64_t> nodes;  // mesh-order node indices
        double v0, v1;
    };
    std::vector<Cond> bcs[4];
    bool bc_dirty = true;

    // materialised boundary conditions
    int nD = 0;
    DevBuf d_didx, d_dval, dmask, inactive_mask;
    bool any_inactive = false;
    SurfaceT<double> s64{};
    SurfaceT<float> s32{};
    DevBuf s_row, s_ptr, s_col, s_val64, s_val32;
    DevBuf smask;  // bit per node: the node has a surface row (CG mode adds k_surface_cg's S x)
    DevBuf splane, smap;  // the TMA operator's surface rows (TmaSurface): plane index, node -> row maps
    TmaSurface tsurf{};
    int rad_rows = 0;
    DevBuf rad_row, rad_ptr, rad_src, rad_coef, rad_tamb;
    int n_fbc = 0;
    DevBuf fbc_idx, fbc_val;

    // masked numbering
    bool masked = false;
    long long n_active = 0;
    DevBuf d_active;                    // canonical index of every masked node, mesh order
    std::vector<long long> h_active;    // same, host
    std::vector<int64_t> h_canon2mask;  // canonical -> masked id (-1 inactive); only when masked

    // parameters
    int algorithm = PLGPU_ALGO_ITERATIVE;
    double rtol = 1e-14;
    int maxit = 0;  // 0: automatic cap
    int noconv = PLGPU_NOCONV_WARNING;
    int empty_mode = PLGPU_EMPTY_DEFAULT;
    int bc_compat = 1;
    double inittemp = 300.0, maxerr = 0.05;
    double inner_rtol = 1e-4;
    bool plain_norm = true;  // PLGPU_NORM_PLAIN: residuals in the 2-norm instead of the Jacobi-scaled norm
    int chunk = 32;

    // time stepping (Dynamic3D): while dyn_active every solve sees theta K + C
    bool dyn_active = false;
    std::vector<double> cp_tab, dens_tab;
    double dyn_dt = 0.1, dyn_theta = 0.5;
    bool dyn_lumping = true;
    int dyn_rebuild = 0, dyn_logfreq = 500;
    double elapstime = 0.0;
    DevBuf d_cp, d_dens, cap64, cap32, kB64, kzB64, Fel, Yb, Zb, Tscratch;
    DevBuf cel64, cel32, celneg64;  // consistent capacity: corner capacity per element, and negated

    // learned preconditioner
    plgpu_unet* pre = nullptr;
    std::unique_ptr<UNetWork> uw;
    DevBuf z32, t32, v32, av32, dscal, dpart;  // z, training scratch, network direction v and A v, scalars
    int fallbacks = 0;
    long long learned_iters = 0;  // CG iterations run with the learned preconditioner

    bool initialized = false;
    int loopno = 0;
    bool converged = true;
    void (*log_cb)(void*, int, const char*) = nullptr;
    void* log_user = nullptr;

    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr, ev3 = nullptr;

    // TMA-staged FP32 CG operator (fem3d_operator_tma.cu) on the direction p32, with its
    // pre-scaled conductances; created on the first coefficient update of a mesh it supports
    TmaOperator* tma = nullptr;
    bool tma_tried = false;
    bool tma_fresh = false;  // tmaP / tmaQ hold the current coefficients
    DevBuf tmaP, tmaQ;
    DevBuf cgpart;  // partial regions of the CG on the TMA operator

    // CUDA graphs of CG chunks: one per (precision, chunk length)
    struct ChunkGraph {
        int len = 0;
        int key = 0;  // 0: FP32 Jacobi-PCG, 1: FP64 Jacobi-PCG, 2: FP32 flexible CG with the network
        cudaGraphExec_t exec = nullptr;
        long long kernels = 0;
    };
    std::vector<ChunkGraph> graphs;
    bool use_graphs = true;

    void invalidate_graphs() {
        for (auto& g : graphs)
            if (g.exec) cudaGraphExecDestroy(g.exec);
        graphs.clear();
    }

    ~plgpu_fem3d() {
        invalidate_graphs();
        if (tma) tma_operator_destroy(tma);
        if (h_ctl) cudaFreeHost(h_ctl);
        for (cudaEvent_t e : {ev0, ev1, ev2, ev3})
            if (e) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }

    void log(int level, const char* fmt, ...) {
        if (!log_cb) return;
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        log_cb(log_user, level, buf);
    }

    // ---------------------------------------------------------------------------------
    // mesh

    // element extent along axis d (a planar mesh has one layer of quads along axis 2)
    int me(int d) const { return (planar && d == 2) ? 1 : n[d] - 1; }

    void setup_mesh(const double* a0, int n0, const double* a1, int n1, const double* a2, int n2, int ord,
                    int plan = 0) {
        const double* a[3] = {a0, a1, a2};
        const int nn[3] = {n0, n1, n2};
        planar = plan;
        for (int d = 0; d < 3; ++d) {
            if (planar && d == 2) {
                ax[2].assign(1, 0.0);
                n[2] = 1;
                continue;
            }
            if (!a[d] || nn[d] < 2) throw ArgError("every axis needs at least 2 nodes");
            ax[d].assign(a[d], a[d] + nn[d]);
            for (int i = 1; i < nn[d]; ++i)
                if (!(ax[d][i] > ax[d][i - 1])) throw ArgError("axis coordinates must be strictly increasing");
            n[d] = nn[d];
        }
        if (ord < 0 || ord > 5) throw ArgError("unknown iteration order");
        static const int orders[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
        ordering = ord;
        major = orders[ord][0];
        medium = orders[ord][1];
        minor = orders[ord][2];
        ns[minor] = 1;
        ns[medium] = n[minor];
        ns[major] = (long long)n[minor] * n[medium];
        es[minor] = 1;
        es[medium] = me(minor);
        es[major] = (long long)me(minor) * me(medium);
        N = (long long)n[0] * n[1] * n[2];
        NE = (long long)me(0) * me(1) * me(2);
        if (N > (1LL << 31) - 1) throw ArgError("meshes above 2^31 nodes are not supported");

        ck(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
        int dev = 0;
        ck(cudaGetDevice(&dev), "cudaGetDevice");
        device = dev;
        ck(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
        noalloc_setup(dev);  // the no-allocation multiply's staging array, looked up here and not in the call
        cfg.stream = stream;
        cfg.sm_count = sm_count;
        if (const char* e = std::getenv("PLGPU_NO_GRAPHS")) use_graphs = !(e[0] == '1');
        prime_launch_shapes();
        cfg.op_share = 1;
        cfg.op_rows = choose_op_rows(n[1]);
        cfg.vec_blocks = sm_count * 4;
        if (cfg.vec_blocks > kMaxPartialBlocks) cfg.vec_blocks = kMaxPartialBlocks;

        for (int d = 0; d < 3; ++d) {
            std::vector<double> h(n[d] - 1), r(n[d] - 1);
            std::vector<float> hf(n[d] - 1), rf(n[d] - 1);
            for (int i = 0; i < n[d] - 1; ++i) {
                h[i] = ax[d][i + 1] - ax[d][i];
                r[i] = 1.0 / h[i];
                hf[i] = (float)h[i];
                rf[i] = (float)r[i];
            }
            upload(h64[d], h, stream);
            upload(r64[d], r, stream);
            upload(h32[d], hf, stream);
            upload(r32[d], rf, stream);
        }
        upload(z64, ax[planar ? 1 : 2], stream);  // coordinates of the vertical axis
        if (planar == PLGPU_GEOMETRY_CYLINDRICAL) {
            if (ax[0][0] < 0.0) throw ArgError("the radial axis of a cylindrical mesh must start at r >= 0");
            std::vector<double> rm((size_t)n[0], 0.0);
            std::vector<float> rmf((size_t)n[0], 0.f);
            for (int i = 0; i < n[0] - 1; ++i) {
                rm[i] = 0.5 * (ax[0][i] + ax[0][i + 1]);  // elem.getMidpoint().rad_r(), therm2d.cpp:333
                rmf[i] = (float)rm[i];
            }
            upload(rmid64, rm, stream);
            upload(rmid32, rmf, stream);
        }
        {
            std::vector<double> zf(n[2] - 1), zr(n[2] - 1);
            std::vector<float> zff(n[2] - 1), zrf(n[2] - 1);
            for (int k = 0; k < n[2] - 1; ++k) {
                const double dz = ax[2][k + 1] - ax[2][k];
                zf[k] = dz / 48.0;
                zr[k] = 1.0 / (48.0 * dz);
                zff[k] = (float)zf[k];
                zrf[k] = (float)zr[k];
            }
            upload(zf64, zf, stream);
            upload(zr64, zr, stream);
            upload(zf32, zff, stream);
            upload(zr32, zrf, stream);
        }
        g64 = GridT<double>{n[0], n[1], n[2], N, h64[0].as<double>(), h64[1].as<double>(), h64[2].as<double>(),
                            r64[0].as<double>(), r64[1].as<double>(), r64[2].as<double>()};
        g32 = GridT<float>{n[0], n[1], n[2], N, h32[0].as<float>(), h32[1].as<float>(), h32[2].as<float>(),
                           r32[0].as<float>(), r32[1].as<float>(), r32[2].as<float>()};

        const size_t N8 = (size_t)N * 8, N4 = (size_t)N * 4;
        T.alloc(N8);
        T0.alloc(N8);
        F.alloc(N8);
        b.alloc(N8);
        r64v.alloc(N8);
        vD.alloc(N8);
        diag.alloc(N8);
        minv64.alloc(N8);
        minv32.alloc(N4);
        k64.alloc(N8);
        k32.alloc(N4);
        p64.alloc(N8);
        q64.alloc(N8);
        x32.alloc(N4);
        r32v.alloc(N4);
        p32.alloc(N4);
        q32.alloc(N4);
        d_mat.alloc((size_t)N * 4);
        d_heat.alloc(N8);
        d_th.alloc(N8);
        const size_t words = (size_t)(N + 31) / 32 + 1;
        dmask.alloc(words * 4);
        inactive_mask.alloc(words * 4);
        partials.alloc(sizeof(double) * kMaxPartialBlocks * 4);
        d_ctl.alloc(sizeof(SolveCtl));
        ck(cudaMemsetAsync(d_ctl.p, 0, sizeof(SolveCtl), stream), "memset");
        ck(cudaMallocHost(&h_ctl, sizeof(SolveCtl)), "cudaMallocHost");
        std::memset(h_ctl, 0, sizeof(SolveCtl));
        for (cudaEvent_t* e : {&ev0, &ev1, &ev2, &ev3}) ck(cudaEventCreate(e), "cudaEventCreate");
        ck(cudaStreamSynchronize(stream), "sync");
    }

    // canonical index of a mesh-order node index
    long long canon_of_mesh(long long m) const {
        const long long imin = m % n[minor];
        const long long imed = (m / n[minor]) % n[medium];
        const long long imaj = m / ((long long)n[minor] * n[medium]);
        long long id[3];
        id[minor] = imin;
        id[medium] = imed;
        id[major] = imaj;
        return id[0] + (long long)n[0] * (id[1] + (long long)n[1] * id[2]);
    }
    long long mesh_of_canon(long long c) const {
        const long long i0 = c % n[0], i1 = (c / n[0]) % n[1], i2 = c / ((long long)n[0] * n[1]);
        return i0 * ns[0] + i1 * ns[1] + i2 * ns[2];
    }

    // ---------------------------------------------------------------------------------
    // inputs

    void set_materials(int nm, const double* k3, const double* pp, const double* kz, const double* he,
                       const uint8_t* em) {
        if (nm <= 0 || !k3 || !pp) throw ArgError("material table needs k300 and p");
        n_mat = nm;
        k300.assign(k3, k3 + nm);
        pexp.assign(pp, pp + nm);
        kzr.assign(nm, 1.0);
        hexp.assign(nm, 0.0);
        empty.assign(nm, 0);
        if (kz) kzr.assign(kz, kz + nm);
        if (he) hexp.assign(he, he + nm);
        if (em) empty.assign(em, em + nm);
        aniso = false;
        for (int m = 0; m < nm; ++m) {
            if (!(k300[m] >= 0.0) || !std::isfinite(k300[m])) throw ArgError("k300 must be finite and >= 0");
            if (kzr[m] != 1.0) aniso = true;
        }
        ktab_T.assign(nm, {});
        ktab_xy.assign(nm, {});
        ktab_z.assign(nm, {});
        any_ktab = false;
        upload(d_k300, k300, stream);
        upload(d_p, pexp, stream);
        upload(d_kzr, kzr, stream);
        upload(d_hexp, hexp, stream);
        if (aniso) {
            kz64.alloc((size_t)N * 8);
            kz32.alloc((size_t)N * 4);
        }
        invalidate_graphs();
        invalidate_solution();
    }

    // A tabulated k(T) for material m (n points; n = 0 removes it), in place of the power law
    void set_material_table(int m, int npts, const double* Tp, const double* kxy, const double* kz) {
        if (n_mat == 0) throw StateError("set the material table first");
        if (m < 0 || m >= n_mat) throw ArgError("material id out of range");
        if (npts < 0) throw ArgError("negative point count");
        if (npts > 0 && (!Tp || !kxy)) throw ArgError("the table needs temperatures and k_xy");
        for (int i = 0; i < npts; ++i) {
            if (!std::isfinite(Tp[i]) || !(Tp[i] > 0.0)) throw ArgError("table temperatures must be finite and > 0");
            if (i > 0 && !(Tp[i] > Tp[i - 1])) throw ArgError("table temperatures must be strictly increasing");
            if (!std::isfinite(kxy[i]) || kxy[i] < 0.0 || (kz && (!std::isfinite(kz[i]) || kz[i] < 0.0)))
                throw ArgError("table conductivities must be finite and >= 0");
        }
        ktab_T[m].assign(Tp, Tp + npts);
        ktab_xy[m].assign(kxy, kxy + npts);
        ktab_z[m].assign(kz ? kz : kxy, (kz ? kz : kxy) + npts);
        // flattened device copy of all tables
        std::vector<int> off((size_t)n_mat, -1), cnt((size_t)n_mat, 0);
        std::vector<double> tT, txy, tz;
        any_ktab = false;
        bool tab_aniso = false;
        for (int q = 0; q < n_mat; ++q) {
            if (ktab_T[q].empty()) continue;
            any_ktab = true;
            off[q] = (int)tT.size();
            cnt[q] = (int)ktab_T[q].size();
            tT.insert(tT.end(), ktab_T[q].begin(), ktab_T[q].end());
            txy.insert(txy.end(), ktab_xy[q].begin(), ktab_xy[q].end());
            tz.insert(tz.end(), ktab_z[q].begin(), ktab_z[q].end());
            for (size_t i = 0; i < ktab_T[q].size(); ++i) tab_aniso |= ktab_z[q][i] != ktab_xy[q][i];
        }
        if (any_ktab) {
            upload(d_toff, off, stream);
            upload(d_tn, cnt, stream);
            upload(d_tT, tT, stream);
            upload(d_txy, txy, stream);
            upload(d_tz, tz, stream);
        }
        bool an = tab_aniso;
        for (int q = 0; q < n_mat; ++q) an |= ktab_T[q].empty() && kzr[q] != 1.0;
        if (an && !aniso) {
            kz64.alloc((size_t)N * 8);
            kz32.alloc((size_t)N * 4);
        }
        aniso = aniso || an;
        bind_tables();
        invalidate_graphs();
        invalidate_solution();
    }
    void bind_tables() {
        tab.tab_off = any_ktab ? d_toff.as<int>() : nullptr;
        tab.tab_n = any_ktab ? d_tn.as<int>() : nullptr;
        tab.tab_T = any_ktab ? d_tT.as<double>() : nullptr;
        tab.tab_kxy = any_ktab ? d_txy.as<double>() : nullptr;
        tab.tab_kz = any_ktab ? d_tz.as<double>() : nullptr;
    }

    void set_elements(const int32_t* mat, const double* heat, const double* leaf) {
        if (!mat) throw ArgError("material ids are required");
        if (n_mat == 0) throw StateError("set the material table first");
        for (long long e = 0; e < NE; ++e)
            if (mat[e] < 0 || mat[e] >= n_mat) throw ArgError("material id out of range");
        host_mat.assign(mat, mat + NE);
        DevBuf tmp;
        tmp.alloc((size_t)NE * 8);
        ck(cudaMemcpyAsync(tmp.p, mat, (size_t)NE * 4, cudaMemcpyHostToDevice, stream), "H2D mat");
        launch_from_mesh_order_i32(cfg, n[0], n[1], n[2], me(0), me(1), me(2), es[0], es[1], es[2],
                                   tmp.as<int>(), d_mat.as<int>(), 0);
        set_heat_impl(heat, tmp);
        if (leaf) {
            d_hleaf.alloc((size_t)N * 8);
            ck(cudaMemcpyAsync(tmp.p, leaf, (size_t)NE * 8, cudaMemcpyHostToDevice, stream), "H2D leaf");
            launch_from_mesh_order_f64(cfg, n[0], n[1], n[2], me(0), me(1), me(2), es[0], es[1], es[2],
                                       tmp.as<double>(), d_hleaf.as<double>(), 0.0);
            have_leaf = true;
        } else {
            have_leaf = false;
        }
        ck(cudaStreamSynchronize(stream), "sync");
        have_elements = true;
        invalidate_solution();
    }

    void set_heat_impl(const double* heat, DevBuf& tmp) {
        if (heat) {
            ck(cudaMemcpyAsync(tmp.p, heat, (size_t)NE * 8, cudaMemcpyHostToDevice, stream), "H2D heat");
            launch_from_mesh_order_f64(cfg, n[0], n[1], n[2], me(0), me(1), me(2), es[0], es[1], es[2],
                                       tmp.as<double>(), d_heat.as<double>(), 0.0);
        } else {
            ck(cudaMemsetAsync(d_heat.p, 0, (size_t)N * 8, stream), "memset");
        }
        heat_dirty = true;
    }

    void set_heat(const double* heat) {
        if (!have_elements) throw StateError("set the elements first");
        DevBuf tmp;
        tmp.alloc((size_t)NE * 8);
        set_heat_impl(heat, tmp);
        ck(cudaStreamSynchronize(stream), "sync");
    }

    void invalidate_solution() {
        initialized = false;
        bc_dirty = true;
        heat_dirty = true;
    }

    // ---------------------------------------------------------------------------------
    // initialisation (onInitialize, therm3d.cpp:71-115; setupMaskedMesh, fem_solver.hpp:182-189)

    bool exclude_empty() const {
        if (empty_mode == PLGPU_EMPTY_INCLUDE) return false;
        if (empty_mode == PLGPU_EMPTY_EXCLUDE) return true;
        return algorithm != PLGPU_ALGO_ITERATIVE;  // reference default: exclude unless iterative
    }

    void initialize() {
        if (n_mat == 0 || !have_elements) throw StateError("materials and elements must be set before computing");
        const bool excl = exclude_empty();
        std::vector<uint8_t> ex(n_mat, 0);
        bool any_ex = false;
        for (int m = 0; m < n_mat; ++m) {
            ex[m] = (excl && empty[m]) ? 1 : 0;
            any_ex |= ex[m] != 0;
        }
        upload(d_excl, ex, stream);
        tab = MatTable{d_k300.as<double>(), d_p.as<double>(), d_kzr.as<double>(), d_hexp.as<double>(),
                       d_excl.as<uint8_t>()};
        bind_tables();

        // masked numbering: nodes touched by an active element, in mesh order
        masked = false;
        any_inactive = false;
        h_active.clear();
        h_canon2mask.clear();
        std::vector<uint32_t> inact((size_t)(N + 31) / 32 + 1, 0u);
        if (any_ex) {
            std::vector<uint8_t> used((size_t)N, 0);
            const int corners = planar ? 4 : 8;
            for (int k = 0; k < me(2); ++k)
                for (int j = 0; j < n[1] - 1; ++j)
                    for (int i = 0; i < n[0] - 1; ++i) {
                        const long long em = i * es[0] + j * es[1] + (long long)k * es[2];
                        if (ex[host_mat[em]]) continue;
                        for (int c = 0; c < corners; ++c) {
                            const long long cn = (i + (c & 1)) + (long long)n[0] * ((j + ((c >> 1) & 1)) +
                                                                                   (long long)n[1] * (k + (c >> 2)));
                            used[cn] = 1;
                        }
                    }
            std::vector<std::pair<long long, long long>> order;  // (mesh index, canonical)
            for (long long cn = 0; cn < N; ++cn) {
                if (used[cn])
                    order.emplace_back(mesh_of_canon(cn), cn);
                else {
                    inact[cn >> 5] |= 1u << (cn & 31);
                    any_inactive = true;
                }
            }
            std::sort(order.begin(), order.end());
            masked = true;
            h_canon2mask.assign((size_t)N, -1);
            h_active.resize(order.size());
            for (size_t t = 0; t < order.size(); ++t) {
                h_active[t] = order[t].second;
                h_canon2mask[order[t].second] = (int64_t)t;
            }
            n_active = (long long)order.size();
            upload(d_active, h_active, stream);
        } else {
            n_active = N;
        }
        upload(inactive_mask, inact, stream);

        // thickness of layer runs
        if (planar)
            launch_thickness2d(cfg, n[0], n[1], d_mat.as<int>(), z64.as<double>(), d_th.as<double>());
        else
            launch_thickness(cfg, n[0], n[1], n[2], d_mat.as<int>(), z64.as<double>(), d_th.as<double>());
        // temperatures = inittemp
        launch_fill(cfg, N, T.as<double>(), inittemp);
        ck(cudaStreamSynchronize(stream), "sync");
        loopno = 0;
        initialized = true;
        bc_dirty = true;
        heat_dirty = true;
    }

    // ---------------------------------------------------------------------------------
    // boundary conditions (setBoundaries, therm3d.cpp:141-168; applyBC, matrix.hpp:111-118)

    bool node_active(long long cn) const { return !masked || h_canon2mask[cn] >= 0; }

    // first matching condition per node (boundary_conditions.hpp:182-186)
    std::unordered_map<long long, int> first_match(int kind) const {
        std::unordered_map<long long, int> m;
        for (size_t c = 0; c < bcs[kind].size(); ++c)
            for (int64_t node : bcs[kind][c].nodes) {
                const long long cn = canon_of_mesh(node);
                if (!node_active(cn)) continue;
                m.emplace(cn, (int)c);
            }
        return m;
    }

    void materialize_bc() {
        invalidate_graphs();  // the surface operator's device arrays are reallocated below
        // Dirichlet set: v_first eliminates, v_last stays in the row (matrix.hpp:132-145)
        std::unordered_map<long long, std::pair<double, double>> dval;
        std::vector<long long> dorder;
        for (const Cond& c : bcs[PLGPU_BC_TEMPERATURE])
            for (int64_t node : c.nodes) {
                const long long cn = canon_of_mesh(node);
                if (!node_active(cn)) continue;
                auto it = dval.find(cn);
                if (it == dval.end()) {
                    dval.emplace(cn, std::make_pair(c.v0, c.v0));
                    dorder.push_back(cn);
                } else {
                    it->second.second = c.v0;
                }
            }
        std::vector<uint32_t> dm((size_t)(N + 31) / 32 + 1, 0u);
        std::vector<int> didx;
        std::vector<double> dv;
        std::vector<double> vfirst_sparse;
        for (long long cn : dorder) {
            dm[cn >> 5] |= 1u << (cn & 31);
            didx.push_back((int)cn);
            dv.push_back(dval[cn].second);
            vfirst_sparse.push_back(dval[cn].first);
        }
        std::vector<int> inactive_nodes;
        if (any_inactive) {
            for (long long cn = 0; cn < N; ++cn)
                if (h_canon2mask[cn] < 0) {
                    dm[cn >> 5] |= 1u << (cn & 31);
                    inactive_nodes.push_back((int)cn);
                }
        }
        auto is_d = [&](long long cn) { return (dm[cn >> 5] >> (cn & 31)) & 1u; };
        nD = (int)didx.size();
        // inactive nodes keep their temperature: treat them as Dirichlet rows at inittemp
        for (int cn : inactive_nodes) {
            didx.push_back(cn);
            dv.push_back(inittemp);
        }
        upload(dmask, dm, stream);
        upload(d_didx, didx, stream);
        upload(d_dval, dv, stream);
        // dense v_first (elimination input)
        ck(cudaMemsetAsync(vD.p, 0, (size_t)N * 8, stream), "memset");
        {
            DevBuf ti, tv;
            std::vector<int> ii(didx.begin(), didx.begin() + nD);
            upload(ti, ii, stream);
            upload(tv, vfirst_sparse, stream);
            launch_scatter_add(cfg, nD, ti.as<int>(), tv.as<double>(), vD.as<double>());
            ck(cudaStreamSynchronize(stream), "sync");
        }

        // face terms
        auto mhf = first_match(PLGPU_BC_HEATFLUX);
        auto mcv = first_match(PLGPU_BC_CONVECTION);
        auto mrd = first_match(PLGPU_BC_RADIATION);
        std::map<long long, double> fadd;                   // static load additions
        std::map<std::pair<long long, long long>, double> K;  // surface stiffness (both triangles)
        struct RadTerm {
            long long row, src;
            double coef, tamb;
        };
        std::vector<RadTerm> rad;

        if (planar) {
            // edge terms of the 2D solvers (setBoundaries, therm2d.cpp:139-172, and its uses
            // at :230-266 Cartesian, :356-407 cylindrical)
            std::vector<long long> cand;
            for (auto* m : {&mhf, &mcv, &mrd})
                for (auto& kv : *m) {
                    const int i = (int)(kv.first % n[0]), j = (int)(kv.first / n[0]);
                    for (int c = 0; c < 4; ++c) {
                        const int e0 = i - (c & 1), e1 = j - (c >> 1);
                        if (e0 < 0 || e1 < 0 || e0 >= n[0] - 1 || e1 >= n[1] - 1) continue;
                        cand.push_back(e0 + (long long)n[0] * e1);
                    }
                }
            std::sort(cand.begin(), cand.end());
            cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
            const bool cyl = planar == PLGPU_GEOMETRY_CYLINDRICAL;
            // the stiffness scale of the edge terms: the reference omits the micrometre
            // factor of len (its load terms carry 0.5e-6) and weights the cylindrical
            // element matrix, edge terms included, by the midpoint radius
            const double kscale = bc_compat ? 1.0 : 1e-6;
            enum { BOTTOM, RIGHT, TOP, LEFT };
            for (long long ec : cand) {
                const int i = (int)(ec % n[0]), j = (int)(ec / n[0]);
                const long long em = i * es[0] + j * es[1];
                const int m = host_mat[em];
                if (exclude_empty() && empty[m]) continue;
                // i1 = lower left, i2 = lower right, i3 = upper right, i4 = upper left
                const long long nd[4] = {ec, ec + 1, ec + 1 + n[0], ec + n[0]};
                const double w = ax[0][i + 1] - ax[0][i], h = ax[1][j + 1] - ax[1][j];
                const double rm = 0.5 * (ax[0][i] + ax[0][i + 1]);
                const double rw = (cyl && bc_compat) ? rm : 1.0;  // the element's weight r K_e
                // edges as (own node, other node, length, side): bottom 1-2, right 2-3, top 3-4, left 1-4
                const int ea[4] = {0, 1, 2, 0}, eb[4] = {1, 2, 3, 3};
                const int sides[4] = {BOTTOM, RIGHT, TOP, LEFT};
                // radius factor of a node's share of an edge term (cylindrical form)
                auto fac = [&](int side, int own, int other, double len) {
                    if (!cyl) return 1.0;
                    if (side == LEFT) return ax[0][i];
                    if (side == RIGHT) return ax[0][i + 1];
                    return rm + (nd[own] < nd[other] ? -len / 6.0 : len / 6.0);
                };
                auto facmn = [&](int side) {
                    if (!cyl) return 1.0;
                    if (side == LEFT) return ax[0][i];
                    if (side == RIGHT) return ax[0][i + 1];
                    return rm;
                };
                for (int kind = PLGPU_BC_HEATFLUX; kind <= PLGPU_BC_RADIATION; ++kind) {
                    auto& mm = kind == PLGPU_BC_HEATFLUX ? mhf : kind == PLGPU_BC_CONVECTION ? mcv : mrd;
                    if (mm.empty()) continue;
                    int cond[4];
                    bool has[4];
                    for (int c = 0; c < 4; ++c) {
                        auto it = mm.find(nd[c]);
                        has[c] = it != mm.end();
                        cond[c] = has[c] ? it->second : -1;
                    }
                    for (int q = 0; q < 4; ++q) {
                        const int a = ea[q], b2 = eb[q];
                        if (!(has[a] && has[b2])) continue;
                        const int side = sides[q];
                        const double len = (side == BOTTOM || side == TOP) ? w : h;
                        const Cond& ca = bcs[kind][cond[a]];
                        const Cond& cb = bcs[kind][cond[b2]];
                        for (int t = 0; t < 2; ++t) {
                            const int own = t ? b2 : a, oth = t ? a : b2;
                            const Cond& co = t ? cb : ca;
                            const double f = fac(side, own, oth, len);
                            if (kind == PLGPU_BC_HEATFLUX) {
                                fadd[nd[own]] += -0.5e-6 * len * co.v0 * f;
                            } else if (kind == PLGPU_BC_CONVECTION) {
                                fadd[nd[own]] += cyl ? 0.125e-6 * len * (ca.v0 + cb.v0) * (ca.v1 + cb.v1) * f
                                                     : 0.5e-6 * len * co.v0 * co.v1;
                                K[{nd[own], nd[own]}] += rw * kscale * (ca.v0 + cb.v0) * len / 6.0 * f;
                            } else {
                                rad.push_back({nd[own], nd[own], -0.5e-6 * len * co.v0 * kSB * f, co.v1});
                            }
                        }
                        if (kind == PLGPU_BC_CONVECTION) {
                            const double v = rw * kscale * (ca.v0 + cb.v0) * len / 12.0 * facmn(side);
                            K[{nd[a], nd[b2]}] += v;
                            K[{nd[b2], nd[a]}] += v;
                        }
                    }
                }
            }
        } else {
            // global nodes 0..7 in the solver's numbering (radiation quirk, therm3d.cpp:265)
            long long glob[8];
            for (int w = 0; w < 8; ++w) {
                long long cn = -1;
                if (masked) {
                    if (w < (long long)h_active.size()) cn = h_active[w];
                } else if (w < N) {
                    cn = canon_of_mesh(w);
                }
                glob[w] = cn;
            }

            std::vector<long long> cand;
            {
                std::vector<long long> nodes;
                for (auto* m : {&mhf, &mcv, &mrd})
                    for (auto& kv : *m) nodes.push_back(kv.first);
                std::vector<long long> els;
                for (long long cn : nodes) {
                    const int i = (int)(cn % n[0]), j = (int)((cn / n[0]) % n[1]), k = (int)(cn / ((long long)n[0] * n[1]));
                    for (int c = 0; c < 8; ++c) {
                        const int e0 = i - (c & 1), e1 = j - ((c >> 1) & 1), e2 = k - (c >> 2);
                        if (e0 < 0 || e1 < 0 || e2 < 0 || e0 >= n[0] - 1 || e1 >= n[1] - 1 || e2 >= n[2] - 1) continue;
                        els.push_back(e0 + (long long)n[0] * (e1 + (long long)n[1] * e2));
                    }
                }
                std::sort(els.begin(), els.end());
                els.erase(std::unique(els.begin(), els.end()), els.end());
                cand.swap(els);
            }
            static const int walls[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 2, 4, 6}, {1, 3, 5, 7}, {0, 1, 4, 5}, {2, 3, 6, 7}};
            for (long long ec : cand) {
                const int i = (int)(ec % n[0]), j = (int)((ec / n[0]) % n[1]), k = (int)(ec / ((long long)n[0] * n[1]));
                const long long em = i * es[0] + j * es[1] + (long long)k * es[2];
                const int m = host_mat[em];
                if (exclude_empty() && empty[m]) continue;
                long long idx[8];
                for (int c = 0; c < 8; ++c)
                    idx[c] = (i + (c & 1)) + (long long)n[0] * ((j + ((c >> 1) & 1)) + (long long)n[1] * (k + (c >> 2)));
                const double dx = ax[0][i + 1] - ax[0][i], dy = ax[1][j + 1] - ax[1][j], dz = ax[2][k + 1] - ax[2][k];
                const double areas[3] = {dx * dy, dy * dz, dz * dx};
                for (int kind = PLGPU_BC_HEATFLUX; kind <= PLGPU_BC_RADIATION; ++kind) {
                    auto& mm = kind == PLGPU_BC_HEATFLUX ? mhf : kind == PLGPU_BC_CONVECTION ? mcv : mrd;
                    if (mm.empty()) continue;
                    int cond[8];
                    bool has[8];
                    for (int c = 0; c < 8; ++c) {
                        auto it = mm.find(idx[c]);
                        has[c] = it != mm.end();
                        cond[c] = has[c] ? it->second : -1;
                    }
                    for (int side = 0; side < 6; ++side) {
                        const int* w = walls[side];
                        if (!(has[w[0]] && has[w[1]] && has[w[2]] && has[w[3]])) continue;
                        const double area = areas[side / 2];
                        for (int a = 0; a < 4; ++a) {
                            const Cond& ca = bcs[kind][cond[w[a]]];
                            // where the term lands: element corner a (reference placement) or the face node
                            const long long ta = bc_compat ? idx[a] : idx[w[a]];
                            if (kind == PLGPU_BC_HEATFLUX) {
                                fadd[ta] += -0.25e-12 * area * ca.v0;
                            } else if (kind == PLGPU_BC_CONVECTION) {
                                fadd[ta] += 0.25e-12 * area * ca.v0 * ca.v1;
                                for (int bq = 0; bq <= a; ++bq) {
                                    const Cond& cb = bcs[kind][cond[w[bq]]];
                                    const int ij = a ^ bq;
                                    const bool edge = (ij == 1 || ij == 2 || ij == 4);
                                    const double v = 0.125e-12 * area * (ca.v0 + cb.v0) / (a == bq ? 9.0 : edge ? 18.0 : 36.0);
                                    const long long tb = bc_compat ? idx[bq] : idx[w[bq]];
                                    K[{ta, tb}] += v;
                                    if (ta != tb) K[{tb, ta}] += v;
                                }
                            } else {
                                const long long src = bc_compat ? glob[w[a]] : idx[w[a]];
                                if (src < 0) throw ArgError("radiation boundary on a mesh with fewer than 8 nodes");
                                rad.push_back({ta, src, -0.25e-12 * area * ca.v0 * kSB, ca.v1});
                            }
                        }
                    }
                }
            }
        }

        // split the surface stiffness: free-free part on the device, free-Dirichlet part
        // eliminated into the static load (b_c -= A(c, r) v_first(r), matrix.hpp:137-144)
        std::vector<int> srow, sptr, scol;
        std::vector<double> sval;
        std::vector<float> sval32;
        long long cur = -1;
        for (auto& kv : K) {
            const long long r = kv.first.first, c = kv.first.second;
            if (is_d(r)) continue;
            if (is_d(c)) {
                auto it = dval.find(c);
                const double v = it != dval.end() ? it->second.first : inittemp;
                fadd[r] -= kv.second * v;
                continue;
            }
            if (r != cur) {
                srow.push_back((int)r);
                sptr.push_back((int)scol.size());
                cur = r;
            }
            scol.push_back((int)c);
            sval.push_back(kv.second);
            sval32.push_back((float)kv.second);
        }
        sptr.push_back((int)scol.size());
        upload(s_row, srow, stream);
        upload(s_ptr, sptr, stream);
        upload(s_col, scol, stream);
        upload(s_val64, sval, stream);
        upload(s_val32, sval32, stream);
        const int nr = (int)srow.size();
        s64 = SurfaceT<double>{nr, s_row.as<int>(), s_ptr.as<int>(), s_col.as<int>(), s_val64.as<double>()};
        s32 = SurfaceT<float>{nr, s_row.as<int>(), s_ptr.as<int>(), s_col.as<int>(), s_val32.as<float>()};
        {
            std::vector<uint32_t> sm((size_t)(N + 31) / 32 + 1, 0u);
            for (int r : srow) sm[(size_t)r >> 5] |= 1u << (r & 31);
            upload(smask, sm, stream);
            // the TMA operator's node -> surface row maps of the planes that hold surface rows
            const long long plane = (long long)n[0] * n[1];
            std::vector<int> sp((size_t)n[2], 0);
            int nplanes = 0;
            for (int r : srow)
                if (sp[(size_t)(r / plane)] == 0) sp[(size_t)(r / plane)] = -1;
            for (int k = 0; k < n[2]; ++k)
                if (sp[k] == -1) sp[k] = ++nplanes;
            std::vector<int> smap_h((size_t)std::max(nplanes, 1) * plane, -1);
            for (size_t q = 0; q < srow.size(); ++q) {
                const long long r = srow[q];
                smap_h[(size_t)(sp[(size_t)(r / plane)] - 1) * plane + (size_t)(r % plane)] = (int)q;
            }
            upload(splane, sp, stream);
            upload(smap, smap_h, stream);
            tsurf = TmaSurface{nplanes > 0 ? splane.as<int>() : nullptr, smap.as<int>(), s_ptr.as<int>(),
                               s_col.as<int>(), s_val32.as<float>()};
        }

        std::vector<int> fi;
        std::vector<double> fv;
        for (auto& kv : fadd) {
            if (is_d(kv.first)) continue;
            fi.push_back((int)kv.first);
            fv.push_back(kv.second);
        }
        n_fbc = (int)fi.size();
        upload(fbc_idx, fi, stream);
        upload(fbc_val, fv, stream);

        std::stable_sort(rad.begin(), rad.end(), [](const RadTerm& a, const RadTerm& b) { return a.row < b.row; });
        std::vector<int> rrow, rptr, rsrc;
        std::vector<double> rcoef, rtamb;
        cur = -1;
        for (const RadTerm& t : rad) {
            if (is_d(t.row)) continue;
            if (t.row != cur) {
                rrow.push_back((int)t.row);
                rptr.push_back((int)rsrc.size());
                cur = t.row;
            }
            rsrc.push_back((int)t.src);
            rcoef.push_back(t.coef);
            rtamb.push_back(t.tamb);
        }
        rptr.push_back((int)rsrc.size());
        rad_rows = (int)rrow.size();
        upload(rad_row, rrow, stream);
        upload(rad_ptr, rptr, stream);
        upload(rad_src, rsrc, stream);
        upload(rad_coef, rcoef, stream);
        upload(rad_tamb, rtamb, stream);
        ck(cudaStreamSynchronize(stream), "sync");
        bc_dirty = false;
        heat_dirty = true;
    }

    void build_static_load() {
        if (planar)
            launch_heat_load2d(cfg, g64, rmid_ptr64(), d_heat.as<double>(), d_mat.as<int>(), tab, F.as<double>());
        else
            launch_heat_load(cfg, g64, d_heat.as<double>(), d_mat.as<int>(), tab, F.as<double>());
        launch_scatter_add(cfg, n_fbc, fbc_idx.as<int>(), fbc_val.as<double>(), F.as<double>());
        heat_dirty = false;
    }

    // ---------------------------------------------------------------------------------
    // the linear solves

    // y = A x (or a variant, see MODE_*) with the optimised operator and the current coefficients
    // MODE_CG: y = A p with the convective surface rows (k_surface_cg first, then the
    // operator), (p, A p) and the step length
    const double* rmid_ptr64() const {
        return planar == PLGPU_GEOMETRY_CYLINDRICAL ? rmid64.as<double>() : nullptr;
    }
    const float* rmid_ptr32() const { return planar == PLGPU_GEOMETRY_CYLINDRICAL ? rmid32.as<float>() : nullptr; }

    // k(T) of every element at the current temperature (setMatrix's thermk calls)
    void update_coef() {
        if (planar)
            launch_coef2d(cfg, n[0], n[1], T.as<double>(), d_mat.as<int>(), d_th.as<double>(), tab, k64.as<double>(),
                          k32.as<float>(), aniso ? kz64.as<double>() : nullptr, aniso ? kz32.as<float>() : nullptr,
                          aniso);
        else
            launch_coef(cfg, n[0], n[1], n[2], T.as<double>(), d_mat.as<int>(), d_th.as<double>(), tab,
                        k64.as<double>(), k32.as<float>(), aniso ? kz64.as<double>() : nullptr,
                        aniso ? kz32.as<float>() : nullptr, aniso);
        refresh_tma();
    }

    // The pre-scaled conductances of the TMA operator from the current FP64 ones; called after
    // every write of k64 / kz64 outside a stream capture.  The first call on a mesh the kernel
    // takes (tma_operator_supported) creates the operator.  Environment: PLGPU_NO_TMA=1 keeps
    // the register-march kernels everywhere; PLGPU_TMA_ALWAYS=1 takes the TMA kernel on every
    // mesh it can run, also where it fills less than 80 % of its columns (tests use it).
    void refresh_tma() {
        tma_fresh = false;
        if (planar) return;
        if (tma && tma_operator_aniso(tma) != aniso) {
            invalidate_graphs();  // captured chunks carry the old operator
            tma_operator_destroy(tma);
            tma = nullptr;
            tma_tried = false;
        }
        if (!tma_tried) {
            tma_tried = true;
            const char* always = std::getenv("PLGPU_TMA_ALWAYS");
            if (std::getenv("PLGPU_NO_TMA") == nullptr &&
                tma_operator_supported(n[0], n[1], n[2], always != nullptr && always[0] == '1')) {
                if (!tmaP.p) tmaP.alloc((size_t)N * 4);
                if (aniso && !tmaQ.p) tmaQ.alloc((size_t)N * 4);
                if (!cgpart.p) cgpart.alloc(sizeof(double) * 3 * kMaxPartialBlocks);
                std::vector<double> hh[3];
                for (int d = 0; d < 3; ++d)
                    for (int i = 0; i + 1 < n[d]; ++i) hh[d].push_back(ax[d][i + 1] - ax[d][i]);
                tma = tma_operator_create(cfg, g64, hh[0], hh[1], hh[2], aniso, p32.as<float>(), tmaP.as<float>(),
                                          aniso ? tmaQ.as<float>() : nullptr);
                if (tma) invalidate_graphs();
            }
        }
        if (!tma) return;
        launch_tma_coef(cfg, tma, g64, k64.as<double>(), aniso ? kz64.as<double>() : nullptr);
        tma_fresh = true;
    }
    // Jacobi diagonal of the current operator and its inverse (FP64 and FP32); `shift` adds
    // the capacity's diagonal of a time step
    void update_diag(const double* shift = nullptr) {
        if (planar) {
            launch_diag2d(cfg, g64, rmid_ptr64(), k64.as<double>(), aniso ? kz64.as<double>() : nullptr,
                          diag.as<double>(), shift);
            launch_finish_diag(cfg, N, s64, dmask.as<uint32_t>(), diag.as<double>(), minv64.as<double>(),
                               minv32.as<float>());
        } else {
            launch_diag(cfg, g64, k64.as<double>(), aniso ? kz64.as<double>() : nullptr, aniso, s64,
                        dmask.as<uint32_t>(), diag.as<double>(), minv64.as<double>(), minv32.as<float>(), shift);
        }
    }

    void op64(const double* x, double* y, const double* rhs, int mode, SolveCtl* ctl = nullptr) {
        SolveCtl* c = ctl ? ctl : d_ctl.as<SolveCtl>();
        int ss = 0;
        if (planar) {
            if (mode == MODE_CG) ss = launch_surface_cg(cfg, s64, x, y, partials.as<double>(), op2d_blocks(cfg, N), c);
            launch_operator2d(cfg, g64, rmid_ptr64(), x, y, k64.as<double>(), aniso ? kz64.as<double>() : nullptr,
                              dmask.as<uint32_t>(), rhs, partials.as<double>(), mode, c,
                              ss > 0 ? smask.as<uint32_t>() : nullptr, ss,
                              dyn_active && dyn_lumping ? cap64.as<double>() : nullptr,
                              dyn_active && !dyn_lumping ? cel64.as<double>() : nullptr);
            return;
        }
        if (mode == MODE_CG)
            ss = launch_surface_cg(cfg, s64, x, y, partials.as<double>(), op_blocks(cfg, n[0], n[1], n[2], true), c);
        launch_operator(cfg, g64, zf64.as<double>(), zr64.as<double>(), x, y, k64.as<double>(),
                        aniso ? kz64.as<double>() : nullptr, aniso, dmask.as<uint32_t>(), rhs, partials.as<double>(),
                        mode, c, ss > 0 ? smask.as<uint32_t>() : nullptr, ss,
                        dyn_active && dyn_lumping ? cap64.as<double>() : nullptr,
                        dyn_active && !dyn_lumping ? cel64.as<double>() : nullptr);
    }
    void op32(const float* x, float* y, int mode, SolveCtl* ctl = nullptr) {
        SolveCtl* c = ctl ? ctl : d_ctl.as<SolveCtl>();
        int ss = 0;
        if (planar) {
            if (mode == MODE_CG) ss = launch_surface_cg(cfg, s32, x, y, partials.as<double>(), op2d_blocks(cfg, N), c);
            launch_operator2d(cfg, g32, rmid_ptr32(), x, y, k32.as<float>(), aniso ? kz32.as<float>() : nullptr,
                              dmask.as<uint32_t>(), (const float*)nullptr, partials.as<double>(), mode, c,
                              ss > 0 ? smask.as<uint32_t>() : nullptr, ss,
                              dyn_active && dyn_lumping ? cap32.as<float>() : nullptr,
                              dyn_active && !dyn_lumping ? cel32.as<float>() : nullptr);
            return;
        }
        if (mode == MODE_CG)
            ss = launch_surface_cg(cfg, s32, x, y, partials.as<double>(), op_blocks(cfg, n[0], n[1], n[2], false), c);
        launch_operator(cfg, g32, zf32.as<float>(), zr32.as<float>(), x, y, k32.as<float>(),
                        aniso ? kz32.as<float>() : nullptr, aniso, dmask.as<uint32_t>(), (const float*)nullptr,
                        partials.as<double>(), mode, c, ss > 0 ? smask.as<uint32_t>() : nullptr, ss,
                        dyn_active && dyn_lumping ? cap32.as<float>() : nullptr,
                        dyn_active && !dyn_lumping ? cel32.as<float>() : nullptr);
    }
    void opR(const double* x, double* y, int mode) { op64(x, y, nullptr, mode); }
    void opR(const float* x, float* y, int mode) { op32(x, y, mode); }

    SolveCtl read_ctl() {
        ck(cudaMemcpyAsync(h_ctl, d_ctl.p, sizeof(SolveCtl), cudaMemcpyDeviceToHost, stream), "D2H ctl");
        ck(cudaStreamSynchronize(stream), "sync");
        return *h_ctl;
    }

    int iteration_cap() const {
        if (maxit > 0) return maxit;
        long long m = 4 * (long long)(n[0] + n[1] + n[2]) * 50;
        return (int)std::min<long long>(std::max<long long>(m, 2000), 200000);
    }

    template <typename R>
    void cg_iterations(const GridT<R>& g, const R* kx, const R* kz, const SurfaceT<R>& s, R* x, R* r, R* p, R* q,
                       const R* minv, int& status, int& iters, int cap) {
        SolveCtl* ctl = d_ctl.as<SolveCtl>();
        double* part = partials.as<double>();
        auto enqueue = [&](int len) {
            for (int it = 0; it < len; ++it) {
                opR(p, q, MODE_CG);
                launch_cg_update(cfg, N, x, r, p, q, minv, part, ctl);
                launch_cg_direction(cfg, N, p, r, minv, ctl);
            }
        };
        run_chunks(sizeof(R) == 8 ? 1 : 0, chunk, 256, enqueue, status, iters, cap);
    }

    // Replay `enqueue(len)` in chunks (captured as CUDA graphs keyed by `key` and
    // length) until the device status word leaves SOLVE_RUNNING or `cap` iterations.
    template <typename F>
    void run_chunks(int key, int first_len, int max_len, F&& enqueue, int& status, int& iters, int cap) {
        int ch = first_len;
        for (;;) {
            if (use_graphs) {
                ChunkGraph* gr = nullptr;
                for (auto& g : graphs)
                    if (g.len == ch && g.key == key) gr = &g;
                if (!gr) {
                    ChunkGraph g;
                    g.len = ch;
                    g.key = key;
                    cudaGraph_t graph = nullptr;
                    ck(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "begin capture");
                    const long long before = thread_launch_count();
                    enqueue(ch);
                    g.kernels = thread_launch_count() - before;
                    count_launches(-g.kernels);  // captured, not run
                    ck(cudaStreamEndCapture(stream, &graph), "end capture");
                    ck(cudaGraphInstantiate(&g.exec, graph, 0), "graph instantiate");
                    cudaGraphDestroy(graph);
                    graphs.push_back(g);
                    gr = &graphs.back();
                }
                ck(cudaGraphLaunch(gr->exec, stream), "graph launch");
                count_launches(gr->kernels);
            } else {
                enqueue(ch);
            }
            ck(cudaGetLastError(), "launch");
            SolveCtl c = read_ctl();
            status = c.status;
            iters = c.iter;
            if (status != SOLVE_RUNNING) return;
            if (c.iter >= cap) return;
            if (ch < max_len) ch *= 2;
        }
    }

    // Convergence of a linear solve.  Residuals are measured in the Jacobi-scaled norm
    // ||r||_{M^-1} = sqrt(sum r_i^2 / A_ii) (Dirichlet rows excluded), which weighs every row
    // against its own diagonal (PLGPU_NORM_SCALED), or in the plain 2-norm over all rows
    // (PLGPU_NORM_PLAIN).  A solve stops when
    //   ||r|| <= rtol ||b||            (FP64 accuracy of the whole solution), and
    //   ||r|| <= kChangeRtol ||r_0||   (the change since the previous solve is resolved:
    //                                   r_0 = b - A T at the start; a small update of the
    //                                   load or of the coefficients moves T by far less
    //                                   than rtol ||b|| would notice),
    // unless that asks for less than the rounding floor of computing b - A T in FP64,
    // estimated as kFloorUlps eps sqrt(sum A_ii T_i^2) (a row sums about 27 products of
    // size A_ii |T|); static solves stop at twice the estimate (one more refinement below
    // it costs 14 % more CG iterations at 128x128x200 and moves max T by < 1e-9 K), time
    // steps, whose right-hand sides carry the capacity terms, at the estimate itself.
    // A solve whose FP64 residual stops falling has reached the floor:
    // it counts as converged when ||r|| <= kStagnationAccept ||b||, as failed above that.
    static constexpr double kChangeRtol = 1e-6;
    static constexpr double kFloorUlps = 8.0;
    static constexpr double kStagnationAccept = 1e-9;

    bool floor_ok(double relres) const { return relres <= std::max(rtol, kStagnationAccept); }

    // weights of the residual norm (nullptr: plain 2-norm); also tells the CG kernels
    const double* norm_weights() {
        ck(cudaMemsetAsync(&d_ctl.as<SolveCtl>()->plain, plain_norm ? 1 : 0, sizeof(int), stream), "memset");
        return plain_norm ? nullptr : minv64.as<double>();
    }

    // relative target of the solve of A T = b from the current T, given ||b||^2 in red[2]
    // and ||r_0||^2 in red[3] (scaled norms); also queues and reads the floor estimate
    double solve_target(double relres0, double bn) {
        launch_diag_norm2(cfg, N, T.as<double>(), minv64.as<double>(), plain_norm ? 1 : 0, partials.as<double>(),
                          d_ctl.as<SolveCtl>(), 4);
        const SolveCtl c = read_ctl();
        const double floor_rel = bn > 0 ? kFloorUlps * 1.1102230246251565e-16 * std::sqrt(c.red[4]) / bn : 0.0;
        return std::max(std::min(rtol, kChangeRtol * relres0), (dyn_active ? 1.0 : 2.0) * floor_rel);
    }

    // FP64 Jacobi-PCG on A T = b starting from the current T.  When the recursive
    // residual reaches the target the true residual is recomputed; CG restarts from
    // the current iterate (at most 3 times) while it is still above twice the target.
    void solve_fp64(int& status, int& iters, double& relres) {
        NvtxRange nv("solve fp64 pcg");
        SolveCtl* ctl = d_ctl.as<SolveCtl>();
        double* part = partials.as<double>();
        const double* w = norm_weights();
        launch_norm2(cfg, N, b.as<double>(), nullptr, part, ctl, 2, w);  // ||b||^2
        residual64();
        launch_norm2(cfg, N, r64v.as<double>(), nullptr, part, ctl, 3, w);
        const SolveCtl c0 = read_ctl();
        const double bn = std::sqrt(c0.red[2]);
        relres = bn > 0 ? std::sqrt(c0.red[3]) / bn : 0.0;
        iters = 0;
        // a NaN or Inf in b or A T fails every comparison: test the norms themselves
        if (!std::isfinite(c0.red[2]) || !std::isfinite(c0.red[3]) || !std::isfinite(relres)) {
            status = SOLVE_NONFINITE;
            return;
        }
        const double target = solve_target(relres, bn);
        if (relres <= target || relres == 0.0) {
            status = SOLVE_CONVERGED;
            return;
        }
        const int cap = iteration_cap();
        const int stall = std::max(500, cap / 10);
        double prev = relres;
        for (int restart = 0; restart < 4; ++restart) {
            int it = 0;
            launch_cg_start(cfg, N, T.as<double>(), false, r64v.as<double>(), p64.as<double>(), minv64.as<double>(),
                            part, ctl, target, 2, cap - iters, stall);
            cg_iterations<double>(g64, k64.as<double>(), aniso ? kz64.as<double>() : nullptr, s64, T.as<double>(),
                                  r64v.as<double>(), p64.as<double>(), q64.as<double>(), minv64.as<double>(), status,
                                  it, cap - iters);
            iters += it;
            residual64();  // true FP64 residual of the iterate
            launch_norm2(cfg, N, r64v.as<double>(), nullptr, part, ctl, 3, w);
            const SolveCtl c = read_ctl();
            relres = bn > 0 ? std::sqrt(c.red[3]) / bn : 0.0;
            if (!std::isfinite(c.red[3])) {
                status = SOLVE_NONFINITE;
                return;
            }
            if (relres <= 2.0 * target) {
                status = SOLVE_CONVERGED;
                return;
            }
            if (status == SOLVE_NONFINITE || status == SOLVE_BREAKDOWN) return;
            if (status == SOLVE_STAGNATED || relres > 0.5 * prev) {  // FP64 rounding floor reached
                status = floor_ok(relres) ? SOLVE_CONVERGED : SOLVE_STAGNATED;
                return;
            }
            if (iters >= cap) {
                status = SOLVE_MAXIT;
                return;
            }
            prev = relres;
        }
        status = floor_ok(relres) ? SOLVE_CONVERGED : SOLVE_MAXIT;
    }

    // The CG of fem3d_cg_fused.cu runs where the TMA operator does
    // the TMA-staged operator is set up for the current coefficients
    bool tma_ready() const { return !planar && tma != nullptr && tma_fresh && !dyn_active; }
    // the inner FP32 solve runs the fused iteration (operator, update, direction): on the
    // TMA-staged operator where it is set up, else on the register-march operator
    bool fused_ready() const {
        static const bool off = std::getenv("PLGPU_NO_FUSED") != nullptr;
        return !planar && !dyn_active && (tma_ready() || !off);
    }
    TmaCg fused_args() {
        if (!cgpart.p) cgpart.alloc(sizeof(double) * 3 * kMaxPartialBlocks);
        const int opb = tma_ready() ? tma_operator_blocks(tma)
                                    : op_blocks(cfg, n[0], n[1], n[2], false) + surface_cg_blocks(s32.nrows);
        return TmaCg{N, x32.as<float>(), r32v.as<float>(), p32.as<float>(), q32.as<float>(), minv32.as<float>(),
                     cgpart.as<double>(), tmacg_blocks(cfg, N), opb};
    }
    // x32 = the FP32 Jacobi-PCG solution of A x = r32v to inner_rtol: the operator with the
    // surface rows (in the TMA kernel, or k_surface_cg before the register-march kernel, its
    // partials after the operator's), then the update and direction kernels
    void fused_cg(int& status, int& iters, int cap) {
        SolveCtl* ctl = d_ctl.as<SolveCtl>();
        const TmaCg f = fused_args();
        const bool staged = tma_ready();
        const int mblocks = staged ? 0 : op_blocks(cfg, n[0], n[1], n[2], false);
        launch_tmacg_start(cfg, f, ctl, inner_rtol, -1, cap, cap);
        auto enqueue = [&](int len) {  // len is even: every chunk starts at parity 0
            for (int it = 0; it < len; ++it) {
                const int q = it & 1;
                const int* run = tmacg_op_run(ctl, q);
                if (staged) {
                    launch_operator_tma(cfg, tma, q32.as<float>(), tmacg_op_partials(f), run, ctl, tsurf);
                } else {
                    const int ss = launch_surface_cg_run(cfg, s32, p32.as<float>(), q32.as<float>(),
                                                         tmacg_op_partials(f), mblocks, run);
                    launch_operator(cfg, g32, zf32.as<float>(), zr32.as<float>(), p32.as<float>(), q32.as<float>(),
                                    k32.as<float>(), aniso ? kz32.as<float>() : nullptr, aniso,
                                    dmask.as<uint32_t>(), (const float*)nullptr, tmacg_op_partials(f), MODE_CG, ctl,
                                    ss > 0 ? smask.as<uint32_t>() : nullptr, ss, nullptr, nullptr, run);
                }
                launch_tmacg_update(cfg, f, ctl, q);
                launch_tmacg_direction(cfg, f, ctl, q);
            }
        };
        run_chunks(staged ? 3 : 4, chunk, 256, enqueue, status, iters, cap);
    }

    // r64 = b - A T (Dirichlet columns eliminated)
    void residual64() {
        op64(T.as<double>(), r64v.as<double>(), b.as<double>(), MODE_RESID);
        launch_surface(cfg, s64, T.as<double>(), r64v.as<double>(), MODE_RESID);
    }

    // FP32 Jacobi-PCG corrections inside FP64 iterative refinement
    void solve_mixed(int& status, int& iters, int& refinements, double& relres) {
        NvtxRange nv("solve mixed");
        SolveCtl* ctl = d_ctl.as<SolveCtl>();
        double* part = partials.as<double>();
        const double* w = norm_weights();
        launch_norm2(cfg, N, b.as<double>(), nullptr, part, ctl, 2, w);
        const int cap = iteration_cap();
        iters = 0;
        refinements = 0;
        status = SOLVE_RUNNING;
        double prev = HUGE_VAL, target = rtol;
        for (int step = 0; step < 60; ++step) {
            residual64();
            launch_norm2(cfg, N, r64v.as<double>(), r32v.as<float>(), part, ctl, 3, w);
            SolveCtl c = read_ctl();
            ++refinements;
            relres = c.red[2] > 0 ? std::sqrt(c.red[3] / c.red[2]) : 0.0;
            if (!std::isfinite(c.red[2]) || !std::isfinite(c.red[3]) || !std::isfinite(relres)) {
                status = SOLVE_NONFINITE;
                return;
            }
            if (step == 0) target = solve_target(relres, std::sqrt(c.red[2]));
            if (relres <= target || relres == 0.0) {
                status = SOLVE_CONVERGED;
                return;
            }
            if (iters >= cap) {
                status = SOLVE_MAXIT;
                return;
            }
            if (step > 2 && relres > 0.5 * prev) {  // refinement no longer contracts: FP64 floor reached
                status = floor_ok(relres) ? SOLVE_CONVERGED : SOLVE_STAGNATED;
                return;
            }
            prev = relres;
            int st = 0, it = 0;
            if (algorithm == PLGPU_ALGO_GPU_LEARNED && pre != nullptr) {
                fcg_inner(st, it, cap - iters);
            } else if (fused_ready()) {
                fused_cg(st, it, cap - iters);
            } else {
                launch_cg_start(cfg, N, x32.as<float>(), true, r32v.as<float>(), p32.as<float>(), minv32.as<float>(),
                                part, ctl, inner_rtol, -1, cap - iters, cap);
                cg_iterations<float>(g32, k32.as<float>(), aniso ? kz32.as<float>() : nullptr, s32, x32.as<float>(),
                                     r32v.as<float>(), p32.as<float>(), q32.as<float>(), minv32.as<float>(), st, it,
                                     cap - iters);
            }
            iters += it;
            if (st == SOLVE_NONFINITE || st == SOLVE_BREAKDOWN || st == SOLVE_DEVICE_TIMEOUT) {
                status = st;
                return;
            }
            launch_add_correction(cfg, N, T.as<double>(), x32.as<float>());
        }
        status = floor_ok(relres) ? SOLVE_CONVERGED : SOLVE_MAXIT;
    }

    // ---------------------------------------------------------------------------------
    // learned preconditioner

    void ensure_unet_buffers() {
        if (!uw) uw.reset(new UNetWork(n[0], n[1], n[2]));
        if (!z32.p) z32.alloc((size_t)N * 4);
        if (!t32.p) t32.alloc((size_t)N * 4);
        if (!v32.p) v32.alloc((size_t)N * 4);
        if (!av32.p) av32.alloc((size_t)N * 4);
        if (!dscal.p) dscal.alloc(64 * 8);
        if (!dpart.p) dpart.alloc((size_t)std::max(8 * sm_count, 4096) * 8);
    }
    void refresh_features() {
        launch_unet_features(cfg, g32, k32.as<float>(), aniso ? kz32.as<float>() : nullptr, aniso, minv32.as<float>(),
                             uw->feat);
    }
    // network direction v = D^-1/2 u(r) into v32, A v into av32, a = (v, r) and b = (v, A v)
    // into dscal[8] and dscal[9]; sigma2 points to (r, D^-1 r) on the device
    void network_direction(const UNetModel& M, const float* r, const double* sigma2) {
        double* sc = dscal.as<double>();
        launch_unet_input(cfg, N, r, minv32.as<float>(), sigma2, uw->feat);
        HeadArgs h = unet_head_args(M, *uw, r, minv32.as<float>(), sigma2, v32.as<float>());
        unet_forward(cfg, M, *uw, &h);
        amul32(v32.as<float>(), av32.as<float>());
        launch_dot(cfg, N, v32.as<float>(), r, dpart.as<double>(), sc + 8);
        launch_dot(cfg, N, v32.as<float>(), av32.as<float>(), dpart.as<double>(), sc + 9);
    }
    // z = P(r) = M^-1 r + c v with c = (v, r) / (v, A v)
    void precond(const UNetModel& M, const float* r, float* z, const double* sigma2) {
        network_direction(M, r, sigma2);
        launch_precond_combine(cfg, N, r, minv32.as<float>(), v32.as<float>(), dscal.as<double>() + 8, z);
    }
    // y = A x with the FP32 system matrix (Dirichlet inputs masked, identity rows)
    void amul32(const float* x, float* y) {
        op32(x, y, MODE_MULT);
        launch_surface(cfg, s32, x, y, MODE_MULT);
    }
    // coefficients and Jacobi at the current temperature (what compute() does per outer loop)
    void prepare_matrix() {
        if (!initialized) initialize();
        if (bc_dirty) materialize_bc();
        launch_coef(cfg, n[0], n[1], n[2], T.as<double>(), d_mat.as<int>(), d_th.as<double>(), tab, k64.as<double>(),
                    k32.as<float>(), aniso ? kz64.as<double>() : nullptr, aniso ? kz32.as<float>() : nullptr, aniso);
        refresh_tma();
        launch_diag(cfg, g64, k64.as<double>(), aniso ? kz64.as<double>() : nullptr, aniso, s64, dmask.as<uint32_t>(),
                    diag.as<double>(), minv64.as<double>(), minv32.as<float>());
        ensure_unet_buffers();
        refresh_features();
    }

    // One training step's forward pass on error e (x32): r = A e, the network direction v,
    // loss L = 1 - a^2 / (b E) (the A-norm error left along v at the optimal weight,
    // relative to e).  Scalars: dscal[0] = (r, D^-1 r), [8] = a = (v, r), [9] = b = (v, A v),
    // [10] = E = (e, A e); z32 receives the full preconditioned residual.
    void loss_forward(const UNetModel& M) {
        double* sc = dscal.as<double>();
        float* e = x32.as<float>();
        float* r = r32v.as<float>();
        amul32(e, r);
        launch_dot(cfg, N, e, r, dpart.as<double>(), sc + 10);
        launch_rmr(cfg, N, r, minv32.as<float>(), dpart.as<double>(), sc + 0);
        network_direction(M, r, sc + 0);
        launch_precond_combine(cfg, N, r, minv32.as<float>(), v32.as<float>(), sc + 8, z32.as<float>());
    }
    void loss_backward(UNetModel& M) {
        double* sc = dscal.as<double>();
        launch_loss_grad_u(cfg, N, r32v.as<float>(), av32.as<float>(), minv32.as<float>(), sc + 8, uw->gu);
        HeadArgs h = unet_head_args(M, *uw, r32v.as<float>(), minv32.as<float>(), sc + 0, v32.as<float>());
        unet_backward(cfg, M, *uw, h);
    }
    static double loss_of(const double* sc) {  // sc = {a, b, E}
        return (sc[1] > 0 && sc[2] > 0) ? 1.0 - sc[0] * sc[0] / (sc[1] * sc[2]) : 1.0;
    }

    // Error of m Jacobi-PCG iterations on A e = 0 started from the noise in x32: the
    // components CG itself removes slowly.
    void cg_smoothed_error(int m) {
        SolveCtl* ctl = d_ctl.as<SolveCtl>();
        amul32(x32.as<float>(), q32.as<float>());
        ck(cudaMemsetAsync(t32.p, 0, (size_t)N * 4, stream), "memset");
        launch_sub(cfg, N, t32.as<float>(), q32.as<float>(), r32v.as<float>());  // r = -A e
        launch_cg_start(cfg, N, x32.as<float>(), false, r32v.as<float>(), p32.as<float>(), minv32.as<float>(),
                        partials.as<double>(), ctl, 0.0, -1, m, m + 1);
        int st = 0, it = 0;
        cg_iterations<float>(g32, k32.as<float>(), aniso ? kz32.as<float>() : nullptr, s32, x32.as<float>(),
                             r32v.as<float>(), p32.as<float>(), q32.as<float>(), minv32.as<float>(), st, it, m);
    }

    // Largest eigenvalue of D^-1 A by 30 power iterations from noise.  On anisotropic
    // layered meshes it reaches 4.5 (thin, wide elements), so a fixed damping such as
    // 0.6 makes "smoothing" sweeps diverge instead of smoothing.
    double jacobi_lambda_max(unsigned long long seed) {
        double* sc = dscal.as<double>();
        launch_noise(cfg, N, seed, minv32.as<float>(), x32.as<float>());
        launch_dot(cfg, N, x32.as<float>(), x32.as<float>(), dpart.as<double>(), sc + 11);
        launch_scale_rms(cfg, N, sc + 11, x32.as<float>());
        double lam = 0.0;
        for (int it = 0; it < 30; ++it) {
            amul32(x32.as<float>(), q32.as<float>());
            ck(cudaMemsetAsync(x32.p, 0, (size_t)N * 4, stream), "memset");
            launch_jacobi_sweep(cfg, N, -1.f, minv32.as<float>(), q32.as<float>(), x32.as<float>());  // D^-1 A x
            launch_dot(cfg, N, x32.as<float>(), x32.as<float>(), dpart.as<double>(), sc + 11);
            double ss = 0.0;
            ck(cudaMemcpyAsync(&ss, sc + 11, 8, cudaMemcpyDeviceToHost, stream), "D2H");
            ck(cudaStreamSynchronize(stream), "sync");
            lam = std::sqrt(ss / (double)N);  // the input had unit RMS
            if (!(lam > 0.0) || !std::isfinite(lam)) break;
            launch_scale_rms(cfg, N, sc + 11, x32.as<float>());
        }
        return lam;
    }

    void train(plgpu_unet* net, int steps, float lr, unsigned long long seed, int smin, int smax, int pair_kind,
               float* losses) {
        if (steps < 0 || !(lr > 0.f) || smin < 0 || smax < smin || pair_kind < 0 || pair_kind > 1)
            throw ArgError("bad training parameters");
        prepare_matrix();
        // damped-Jacobi smoothing with omega lambda_max = 1.2 (the power iteration
        // approaches lambda_max from below; 1.2 keeps a 40 % margin to divergence at 2)
        const double lmax = pair_kind == 0 ? jacobi_lambda_max(seed ^ 0x5DEECE66Dull) : 1.0;
        const float omega = (float)(lmax > 0.0 ? 1.2 / lmax : 0.6);
        log(5, "training pairs: lambda_max(D^-1 A) ~ %g, Jacobi damping %g", lmax, (double)omega);
        DevBuf dl;
        dl.alloc((size_t)std::max(steps, 1) * 3 * 8);
        double* sc = dscal.as<double>();
        for (int st = 0; st < steps; ++st) {
            unsigned long long h = (seed + 1) * 0x9E3779B97F4A7C15ull + (unsigned long long)st * 0xBF58476D1CE4E5B9ull;
            h ^= h >> 31;
            const int m = smin + (int)(h % (unsigned long long)(smax - smin + 1));
            launch_noise(cfg, N, h, minv32.as<float>(), x32.as<float>());
            if (pair_kind == 0) {
                for (int q = 0; q < m; ++q) {
                    amul32(x32.as<float>(), q32.as<float>());
                    launch_jacobi_sweep(cfg, N, omega, minv32.as<float>(), q32.as<float>(), x32.as<float>());
                }
            } else if (m > 0) {
                cg_smoothed_error(m);
            }
            launch_dot(cfg, N, x32.as<float>(), x32.as<float>(), dpart.as<double>(), sc + 11);
            launch_scale_rms(cfg, N, sc + 11, x32.as<float>());  // unit RMS keeps BF16 ranges comfortable
            loss_forward(net->model);
            ck(cudaMemcpyAsync(dl.as<double>() + 3 * st, sc + 8, 3 * 8, cudaMemcpyDeviceToDevice, stream), "copy");
            loss_backward(net->model);
            unet_adam(cfg, net->model, lr);
        }
        ck(cudaGetLastError(), "launch");
        std::vector<double> hl((size_t)steps * 3);
        if (steps) ck(cudaMemcpyAsync(hl.data(), dl.p, hl.size() * 8, cudaMemcpyDeviceToHost, stream), "D2H");
        ck(cudaStreamSynchronize(stream), "sync");
        if (losses)
            for (int st = 0; st < steps; ++st) losses[st] = (float)loss_of(&hl[3 * st]);
    }

    // full node array (mesh order, double) -> canonical FP32 in dst
    void host_to_f32(const double* in, float* dst) {
        DevBuf tmp;
        tmp.alloc((size_t)N * 8);
        ck(cudaMemcpyAsync(tmp.p, in, (size_t)N * 8, cudaMemcpyHostToDevice, stream), "H2D");
        launch_from_mesh_order_f64(cfg, n[0], n[1], n[2], n[0], n[1], n[2], ns[0], ns[1], ns[2], tmp.as<double>(),
                                   p64.as<double>(), 0.0);
        launch_norm2(cfg, N, p64.as<double>(), dst, partials.as<double>(), d_ctl.as<SolveCtl>(), 4);
        ck(cudaStreamSynchronize(stream), "sync");
    }
    void f32_to_host(const float* src, double* out) {
        DevBuf tmp;
        tmp.alloc((size_t)N * 8);
        launch_widen(cfg, N, src, q64.as<double>());
        launch_to_mesh_order_f64(cfg, n[0], n[1], n[2], n[0], (long long)n[0] * n[1], ns[0], ns[1], ns[2], 1,
                                 q64.as<double>(), tmp.as<double>());
        ck(cudaMemcpyAsync(out, tmp.p, (size_t)N * 8, cudaMemcpyDeviceToHost, stream), "D2H");
        ck(cudaStreamSynchronize(stream), "sync");
    }

    void loss_grad(plgpu_unet* net, const double* e, double* loss, float* grad, double* r_out, double* z_out) {
        prepare_matrix();
        host_to_f32(e, x32.as<float>());
        loss_forward(net->model);
        ck(cudaMemsetAsync(net->model.g, 0, net->model.n_params * 4, stream), "memset");
        loss_backward(net->model);
        double sc[3];
        ck(cudaMemcpyAsync(sc, dscal.as<double>() + 8, 3 * 8, cudaMemcpyDeviceToHost, stream), "D2H");
        ck(cudaMemcpyAsync(grad, net->model.g, net->model.n_params * 4, cudaMemcpyDeviceToHost, stream), "D2H");
        ck(cudaStreamSynchronize(stream), "sync");
        *loss = loss_of(sc);
        if (r_out) f32_to_host(r32v.as<float>(), r_out);
        if (z_out) f32_to_host(z32.as<float>(), z_out);
    }

    void apply_net(plgpu_unet* net, const double* r, double* z) {
        prepare_matrix();
        host_to_f32(r, r32v.as<float>());
        launch_rmr(cfg, N, r32v.as<float>(), minv32.as<float>(), dpart.as<double>(), dscal.as<double>());
        precond(net->model, r32v.as<float>(), z32.as<float>(), dscal.as<double>());
        f32_to_host(z32.as<float>(), z);
    }

    // Device time (CUDA events on the solver's stream, averaged over reps after one untimed
    // pass) of one network forward pass (input scaling, the U-Net, the head) and of one whole
    // preconditioner application (forward, A v, (v, r), (v, A v), z = M^-1 r + c v), on a
    // residual of ones at the current temperature's matrix.
    void time_net(plgpu_unet* net, int reps, double* fwd_ms, double* pre_ms) {
        if (reps <= 0) throw ArgError("reps must be positive");
        prepare_matrix();
        std::vector<double> ones((size_t)N, 1.0);
        host_to_f32(ones.data(), r32v.as<float>());
        double* sc = dscal.as<double>();
        launch_rmr(cfg, N, r32v.as<float>(), minv32.as<float>(), dpart.as<double>(), sc);
        const UNetModel& M = net->model;
        float tf = 0.f, tp = 0.f;
        for (int k = -1; k < reps; ++k) {
            float a = 0.f, b2 = 0.f;
            ck(cudaEventRecord(ev2, stream), "event");
            launch_unet_input(cfg, N, r32v.as<float>(), minv32.as<float>(), sc, uw->feat);
            HeadArgs h = unet_head_args(M, *uw, r32v.as<float>(), minv32.as<float>(), sc, v32.as<float>());
            unet_forward(cfg, M, *uw, &h);
            ck(cudaEventRecord(ev3, stream), "event");
            ck(cudaEventSynchronize(ev3), "sync");
            ck(cudaEventElapsedTime(&a, ev2, ev3), "elapsed");
            ck(cudaEventRecord(ev2, stream), "event");
            precond(M, r32v.as<float>(), z32.as<float>(), sc);
            ck(cudaEventRecord(ev3, stream), "event");
            ck(cudaEventSynchronize(ev3), "sync");
            ck(cudaEventElapsedTime(&b2, ev2, ev3), "elapsed");
            if (k >= 0) {
                tf += a;
                tp += b2;
            }
        }
        ck(cudaGetLastError(), "launch");
        *fwd_ms = tf / reps;
        *pre_ms = tp / reps;
    }

    // Inner FP32 solve with flexible CG and the network; Jacobi-PCG takes over from the
    // current iterate when the flexible CG stagnates or breaks down.
    void fcg_inner(int& st, int& it, int cap) {
        SolveCtl* ctl = d_ctl.as<SolveCtl>();
        double* part = partials.as<double>();
        const UNetModel& M = pre->model;
        float *x = x32.as<float>(), *r = r32v.as<float>(), *p = p32.as<float>(), *q = q32.as<float>(),
              *z = z32.as<float>();
        const float* minv = minv32.as<float>();
        launch_cg_start(cfg, N, x, true, r, p, minv, part, ctl, inner_rtol, 3, cap, 40);
        precond(M, r, z, &ctl->rz);
        launch_fcg_dots(cfg, N, z, r, q, part, ctl, 1);
        launch_fcg_direction(cfg, N, p, z, ctl);
        auto enqueue = [&](int len) {
            for (int k = 0; k < len; ++k) {
                op32(p, q, MODE_CG);
                launch_cg_update(cfg, N, x, r, p, q, minv, part, ctl);
                precond(M, r, z, &ctl->rz);
                launch_fcg_dots(cfg, N, z, r, q, part, ctl, 0);
                launch_fcg_direction(cfg, N, p, z, ctl);
            }
        };
        run_chunks(2, 4, 16, enqueue, st, it, cap);
        learned_iters += it;
        if (st == SOLVE_STAGNATED || st == SOLVE_BREAKDOWN || (st == SOLVE_MAXIT && it < cap)) {
            ++fallbacks;
            int st2 = 0, it2 = 0;
            launch_cg_start(cfg, N, x, false, r, p, minv, part, ctl, inner_rtol, 3, cap - it, cap);
            cg_iterations<float>(g32, k32.as<float>(), aniso ? kz32.as<float>() : nullptr, s32, x, r, p, q, minv, st2,
                                 it2, cap - it);
            st = st2;
            it += it2;
        }
    }

    // ---------------------------------------------------------------------------------
    // compute (therm3d.cpp:281-340)

    double compute(int loops, plgpu_stats* st) {
        NvtxRange nv("thermal compute");
        if (!initialized) initialize();
        if (bc_dirty) materialize_bc();
        const long long launches0 = thread_launch_count();
        const int fallbacks0 = fallbacks;
        const long long learned0 = learned_iters;
        ck(cudaEventRecord(ev0, stream), "event");
        if (heat_dirty) build_static_load();
        log(3, "Running thermal calculations");
        double toterr = 0.0, err = 0.0, maxT = 0.0, relres = 0.0;
        int loop = 0, total_iters = 0, total_ref = 0;
        float solve_ms = 0.f;
        const bool mixed = algorithm == PLGPU_ALGO_ITERATIVE || algorithm == PLGPU_ALGO_GPU_MIXED ||
                           algorithm == PLGPU_ALGO_GPU_LEARNED;
        do {
            NvtxRange nv_loop("outer loop");
            ck(cudaMemcpyAsync(T0.p, T.p, (size_t)N * 8, cudaMemcpyDeviceToDevice, stream), "copy T0");
            // setMatrix: coefficients, Jacobi diagonal, right-hand side with Dirichlet elimination
            {
                NvtxRange nv_set("setMatrix");
                update_coef();
                update_diag();
                if (algorithm == PLGPU_ALGO_GPU_LEARNED && pre != nullptr) {
                    ensure_unet_buffers();
                    refresh_features();
                }
                op64(vD.as<double>(), b.as<double>(), F.as<double>(), MODE_RHS);
                launch_radiation(cfg, rad_rows, rad_row.as<int>(), rad_ptr.as<int>(), rad_src.as<int>(),
                                 rad_coef.as<double>(), rad_tamb.as<double>(), T.as<double>(), b.as<double>());
                launch_set_dirichlet(cfg, (int)(d_didx.bytes / sizeof(int)), d_didx.as<int>(), d_dval.as<double>(),
                                     b.as<double>(), T.as<double>());
                ck(cudaGetLastError(), "launch");
            }
            ck(cudaEventRecord(ev2, stream), "event");
            int status = 0, iters = 0, refs = 0;
            if (mixed)
                solve_mixed(status, iters, refs, relres);
            else
                solve_fp64(status, iters, relres);
            ck(cudaEventRecord(ev3, stream), "event");
            total_iters += iters;
            total_ref += refs;
            if (status == SOLVE_DEVICE_TIMEOUT)
                throw SolveError(PLGPU_ERR_CUDA, "a device-side wait for staged copies timed out");
            if (status == SOLVE_NONFINITE)
                throw SolveError(PLGPU_ERR_NONFINITE, "non-finite value in the linear solve");
            if (status == SOLVE_BREAKDOWN)
                throw SolveError(PLGPU_ERR_NOT_SPD, "stiffness matrix is not positive definite (CG breakdown)");
            converged = status == SOLVE_CONVERGED;
            if (!converged) {
                if (noconv == PLGPU_NOCONV_ERROR)
                    throw SolveError(PLGPU_ERR_NOCONV, "failed to converge in " + std::to_string(iters) +
                                                           " iterations (relative residual " +
                                                           std::to_string(relres) + ")");
                log(noconv == PLGPU_NOCONV_WARNING ? 2 : 5, "Failed to converge in %d iterations (error %g)", iters,
                    relres);
            }
            launch_err(cfg, N, T.as<double>(), T0.as<double>(), any_inactive ? inactive_mask.as<uint32_t>() : nullptr,
                       partials.as<double>(), d_ctl.as<SolveCtl>());
            SolveCtl c = read_ctl();
            float ms = 0.f;
            ck(cudaEventElapsedTime(&ms, ev2, ev3), "elapsed");
            solve_ms += ms;
            err = c.red[0];
            maxT = c.red[1] > 0 ? c.red[1] : 0.0;
            if (err > toterr) toterr = err;
            ++loopno;
            ++loop;
            log(4, "Loop %d(%d): max(T) = %.3f K, error = %g K", loop, loopno, maxT, err);
            if (loop >= kMaxOuterLoops) break;
        } while ((!converged || err > maxerr) && (loops == 0 || loop < loops));
        ck(cudaEventRecord(ev1, stream), "event");
        ck(cudaEventSynchronize(ev1), "sync");
        float tot = 0.f;
        ck(cudaEventElapsedTime(&tot, ev0, ev1), "elapsed");
        if (st) {
            st->loops = loop;
            st->total_loops = loopno;
            st->inner_iterations = total_iters;
            st->refinements = total_ref;
            st->converged = converged ? 1 : 0;
            st->fallbacks = fallbacks - fallbacks0;
            st->learned_iterations = (int)(learned_iters - learned0);
            st->err = err;
            st->toterr = toterr;
            st->max_t = maxT;
            st->last_rel_residual = relres;
            st->solve_ms = solve_ms;
            st->total_ms = tot;
            st->kernel_launches = thread_launch_count() - launches0;
        }
        return toterr;
    }

    // ---------------------------------------------------------------------------------
    // Dynamic3D (solvers/thermal/dynamic/femT3d.cpp): theta-method time stepping with the
    // lumped heat capacity.  setMatrix builds A = theta K + C (K scaled in place, C as the
    // operator's diagonal shift), keeps the unscaled K for B = C - (1 - theta) K and the
    // load F with A's Dirichlet elimination (femT3d.cpp:128-252); every step solves
    // A T' = B T + F with the Dirichlet rows of the right-hand side (and of T) set to their
    // values, the theta method that setMatrix prepares.  (The reference's step loop,
    // femT3d.cpp:291-300, adds (B T)[r] to those rows, B never getting the boundary
    // conditions, and passes the vectors through buffers that alias after the first
    // step; on meshes whose capacity per node exceeds 1 that grows without bound.)

    // lumped capacity per node (weight x the corner capacities around it) and the
    // consistent matrix's corner capacity per element; 3D hexes or planar quads
    void lumped_capacity(double* c64, float* c32, double weight) {
        if (planar)
            launch_lumped_mass2d(cfg, g64, rmid_ptr64(), d_mat.as<int>(), d_excl.as<uint8_t>(), d_cp.as<double>(),
                                 d_dens.as<double>(), dyn_dt, c64, c32, weight);
        else
            launch_lumped_mass(cfg, g64, d_mat.as<int>(), d_excl.as<uint8_t>(), d_cp.as<double>(),
                               d_dens.as<double>(), dyn_dt, c64, c32, weight);
    }
    void element_capacity() {
        if (planar)
            launch_elem_capacity2d(cfg, g64, rmid_ptr64(), d_mat.as<int>(), d_excl.as<uint8_t>(), d_cp.as<double>(),
                                   d_dens.as<double>(), dyn_dt, cel64.as<double>(), cel32.as<float>(),
                                   celneg64.as<double>());
        else
            launch_elem_capacity(cfg, g64, d_mat.as<int>(), d_excl.as<uint8_t>(), d_cp.as<double>(),
                                 d_dens.as<double>(), dyn_dt, cel64.as<double>(), cel32.as<float>(),
                                 celneg64.as<double>());
    }
    // y = rhs - (kB x + cneg-capacity x), the right-hand side product of a time step
    void op_step_rhs(const double* x, double* y, const double* rhs, const double* cneg) {
        if (planar)
            launch_operator2d(cfg, g64, rmid_ptr64(), x, y, kB64.as<double>(), aniso ? kzB64.as<double>() : nullptr,
                              dmask.as<uint32_t>(), rhs, partials.as<double>(), MODE_RHS, d_ctl.as<SolveCtl>(),
                              nullptr, 0, nullptr, cneg);
        else
            launch_operator(cfg, g64, zf64.as<double>(), zr64.as<double>(), x, y, kB64.as<double>(),
                            aniso ? kzB64.as<double>() : nullptr, aniso, dmask.as<uint32_t>(), rhs,
                            partials.as<double>(), MODE_RHS, d_ctl.as<SolveCtl>(), nullptr, 0, nullptr, cneg);
    }

    void dyn_set_matrix() {
        const size_t N8 = (size_t)N * 8;
        update_coef();
        ck(cudaMemcpyAsync(kB64.p, k64.p, N8, cudaMemcpyDeviceToDevice, stream), "copy k");
        if (aniso) ck(cudaMemcpyAsync(kzB64.p, kz64.p, N8, cudaMemcpyDeviceToDevice, stream), "copy kz");
        launch_scale4(cfg, N, dyn_theta, k64.as<double>(), k32.as<float>(), aniso ? kz64.as<double>() : nullptr,
                      aniso ? kz32.as<float>() : nullptr);
        refresh_tma();
        if (dyn_lumping) {
            lumped_capacity(cap64.as<double>(), cap32.as<float>(), 1.0);
        } else {
            // consistent C: corner capacities for the operator, its diagonal ((2/3)^3 = 8/27 c
            // per hex corner, (2/3)^2 = 4/9 c per quad corner) for the Jacobi preconditioner,
            // and B's stiffness part (1 - theta) K kept in kB for the right-hand side product
            element_capacity();
            lumped_capacity(cap64.as<double>(), nullptr, planar ? 4.0 / 9.0 : 8.0 / 27.0);
            launch_scale4(cfg, N, 1.0 - dyn_theta, kB64.as<double>(), nullptr, aniso ? kzB64.as<double>() : nullptr,
                          nullptr);
        }
        update_diag(cap64.as<double>());
        // F with the elimination of A's Dirichlet columns, the row values at the Dirichlet rows
        op64(vD.as<double>(), Fel.as<double>(), F.as<double>(), MODE_RHS);
        launch_set_dirichlet(cfg, (int)(d_didx.bytes / sizeof(int)), d_didx.as<int>(), d_dval.as<double>(),
                             Fel.as<double>(), Tscratch.as<double>());
    }

    double compute_dynamic(double time, plgpu_stats* st) {
        NvtxRange nv("time stepping");
        if (cp_tab.empty()) throw StateError("set the heat capacities first (plgpu_fem3d_set_dynamic)");
        for (int kind = 1; kind < 4; ++kind)
            if (!bcs[kind].empty())
                throw ArgError("the time-stepping solver takes temperature boundary conditions only");
        if (!initialized) {
            initialize();
            elapstime = 0.0;  // onInitialize, femT3d.cpp:77-81
        }
        if (bc_dirty) materialize_bc();
        const size_t N8 = (size_t)N * 8;
        kB64.alloc(N8);
        if (aniso) kzB64.alloc(N8);
        cap64.alloc(N8);
        cap32.alloc((size_t)N * 4);
        if (!dyn_lumping) {
            cel64.alloc(N8);
            cel32.alloc((size_t)N * 4);
            celneg64.alloc(N8);
        }
        Fel.alloc(N8);
        Yb.alloc(N8);
        Tscratch.alloc(N8);
        if (Zb.bytes != N8) {
            Zb.alloc(N8);
            ck(cudaMemsetAsync(Zb.p, 0, N8, stream), "memset");
        }
        upload(d_cp, cp_tab, stream);
        upload(d_dens, dens_tab, stream);
        const long long launches0 = thread_launch_count();
        const int fallbacks0 = fallbacks;
        const long long learned0 = learned_iters;
        ck(cudaEventRecord(ev0, stream), "event");
        if (heat_dirty) build_static_load();
        invalidate_graphs();  // captured solves carry the operator without the capacity shift
        // The capacity terms C T dominate ||b|| while the smallest elements carry the
        // smallest rows of A: the time steps measure residuals in the Jacobi-scaled norm.
        struct Guard {
            plgpu_fem3d* h;
            bool plain;
            ~Guard() {
                h->dyn_active = false;
                h->plain_norm = plain;
                h->invalidate_graphs();
            }
        } guard{this, plain_norm};
        dyn_active = true;
        plain_norm = false;
        log(3, "Running thermal calculations");
        dyn_set_matrix();
        const bool mixed = algorithm == PLGPU_ALGO_ITERATIVE || algorithm == PLGPU_ALGO_GPU_MIXED ||
                           algorithm == PLGPU_ALGO_GPU_LEARNED;
        const int nrows = (int)(d_didx.bytes / sizeof(int));
        long long r = dyn_rebuild, l = dyn_logfreq;
        int total_iters = 0, total_ref = 0, steps = 0;
        double relres = 0.0, maxT = 0.0;
        float solve_ms = 0.f;
        time += dyn_dt / 2.0;
        for (double t = 0.0; t < time; t += dyn_dt) {
            NvtxRange nv_step("time step");
            if (dyn_rebuild && r == 0) {
                dyn_set_matrix();
                r = dyn_rebuild;
            }
            // X = B T + F = C T - (1 - theta) K T + F, then Dirichlet rows of T take X
            if (dyn_lumping) {
                op_step_rhs(T.as<double>(), Yb.as<double>(), Zb.as<double>(), nullptr);
                launch_dyn_rhs(cfg, N, cap64.as<double>(), T.as<double>(), Yb.as<double>(), 1.0 - dyn_theta,
                               Fel.as<double>(), b.as<double>());
            } else {
                // one operator pass: F - ((1 - theta) K - C) T with kB = (1 - theta) K and -c
                op_step_rhs(T.as<double>(), b.as<double>(), Fel.as<double>(), celneg64.as<double>());
            }
            launch_set_dirichlet(cfg, nrows, d_didx.as<int>(), d_dval.as<double>(), b.as<double>(), T.as<double>());
            ck(cudaEventRecord(ev2, stream), "event");
            int status = 0, iters = 0, refs = 0;
            if (mixed)
                solve_mixed(status, iters, refs, relres);
            else
                solve_fp64(status, iters, relres);
            ck(cudaEventRecord(ev3, stream), "event");
            total_iters += iters;
            total_ref += refs;
            if (status == SOLVE_DEVICE_TIMEOUT)
                throw SolveError(PLGPU_ERR_CUDA, "a device-side wait for staged copies timed out");
            if (status == SOLVE_NONFINITE) throw SolveError(PLGPU_ERR_NONFINITE, "non-finite value in the linear solve");
            if (status == SOLVE_BREAKDOWN)
                throw SolveError(PLGPU_ERR_NOT_SPD, "system matrix is not positive definite (CG breakdown)");
            converged = status == SOLVE_CONVERGED;
            if (!converged) {
                if (noconv == PLGPU_NOCONV_ERROR)
                    throw SolveError(PLGPU_ERR_NOCONV, "failed to converge in " + std::to_string(iters) +
                                                           " iterations (relative residual " +
                                                           std::to_string(relres) + ")");
                log(noconv == PLGPU_NOCONV_WARNING ? 2 : 5, "Failed to converge in %d iterations (error %g)", iters,
                    relres);
            }
            float ms = 0.f;
            ck(cudaEventSynchronize(ev3), "sync");
            ck(cudaEventElapsedTime(&ms, ev2, ev3), "elapsed");
            solve_ms += ms;
            if (dyn_logfreq && l == 0) {
                launch_err(cfg, N, T.as<double>(), T.as<double>(),
                           any_inactive ? inactive_mask.as<uint32_t>() : nullptr, partials.as<double>(),
                           d_ctl.as<SolveCtl>());
                maxT = read_ctl().red[1];
                log(4, "Time %.2f ns: max(T) = %.3f K", elapstime, maxT);
                l = dyn_logfreq;
            }
            --r;
            --l;
            elapstime += dyn_dt;
            ++steps;
        }
        elapstime -= dyn_dt;
        launch_err(cfg, N, T.as<double>(), T.as<double>(), any_inactive ? inactive_mask.as<uint32_t>() : nullptr,
                   partials.as<double>(), d_ctl.as<SolveCtl>());
        maxT = read_ctl().red[1];
        ck(cudaEventRecord(ev1, stream), "event");
        ck(cudaEventSynchronize(ev1), "sync");
        float tot = 0.f;
        ck(cudaEventElapsedTime(&tot, ev0, ev1), "elapsed");
        ++loopno;
        if (st) {
            st->loops = steps;
            st->total_loops = loopno;
            st->inner_iterations = total_iters;
            st->refinements = total_ref;
            st->converged = converged ? 1 : 0;
            st->fallbacks = fallbacks - fallbacks0;
            st->learned_iterations = (int)(learned_iters - learned0);
            st->err = 0.0;
            st->toterr = 0.0;
            st->max_t = maxT;
            st->last_rel_residual = relres;
            st->solve_ms = solve_ms;
            st->total_ms = tot;
            st->kernel_launches = thread_launch_count() - launches0;
        }
        return 0.0;  // femT3d.cpp:314
    }

    // ---------------------------------------------------------------------------------
    // timing of the operator kernel (the CG-mode stencil application) on the current state

    void time_operator(int precision, int reps, int flush_l2, double* avg_ms, double* bytes) {
        if (!initialized) initialize();
        if (bc_dirty) materialize_bc();
        if (reps <= 0) throw ArgError("reps must be positive");
        // coefficients of the current temperature, a deterministic input vector
        update_coef();
        launch_fill(cfg, N, p64.as<double>(), 1.0);
        launch_norm2(cfg, N, p64.as<double>(), p32.as<float>(), partials.as<double>(), d_ctl.as<SolveCtl>(), 4);
        // a scratch control block: the CG-mode operator sets a step length and may flag a
        // breakdown for this synthetic input, which must not stop the next repetition
        DevBuf scratch;
        scratch.alloc(sizeof(SolveCtl));
        SolveCtl* ctl = scratch.as<SolveCtl>();
        ck(cudaMemsetAsync(ctl, 0, sizeof(SolveCtl), stream), "memset");  // SOLVE_RUNNING, counters 0
        DevBuf flush;
        if (flush_l2) flush.alloc((size_t)512 << 20);  // well above the 126 MiB L2
        float total = 0.f;
        // two untimed launches first: the first launch of a kernel in a process also loads it
        for (int r = -2; r < reps; ++r) {
            if (flush_l2) ck(cudaMemsetAsync(flush.p, r & 0xff, flush.bytes, stream), "flush");
            ck(cudaMemsetAsync(&ctl->status, 0, sizeof(int), stream), "memset");
            ck(cudaEventRecord(ev2, stream), "event");
            // the stencil kernel alone (no surface rows)
            if (planar && precision == 64)
                launch_operator2d(cfg, g64, rmid_ptr64(), p64.as<double>(), q64.as<double>(), k64.as<double>(),
                                  aniso ? kz64.as<double>() : nullptr, dmask.as<uint32_t>(), (const double*)nullptr,
                                  partials.as<double>(), MODE_CG, ctl, nullptr, 0);
            else if (planar)
                launch_operator2d(cfg, g32, rmid_ptr32(), p32.as<float>(), q32.as<float>(), k32.as<float>(),
                                  aniso ? kz32.as<float>() : nullptr, dmask.as<uint32_t>(), (const float*)nullptr,
                                  partials.as<double>(), MODE_CG, ctl, nullptr, 0);
            else if (precision == 64)
                launch_operator(cfg, g64, zf64.as<double>(), zr64.as<double>(), p64.as<double>(), q64.as<double>(),
                                k64.as<double>(), aniso ? kz64.as<double>() : nullptr, aniso, dmask.as<uint32_t>(),
                                nullptr, partials.as<double>(), MODE_CG, ctl);
            else if (tma_ready())  // the kernel the FP32 CG solve runs, without surface rows
                launch_operator_tma(cfg, tma, q32.as<float>(), partials.as<double>(), &ctl->status, ctl,
                                    TmaSurface{});
            else
                launch_operator(cfg, g32, zf32.as<float>(), zr32.as<float>(), p32.as<float>(), q32.as<float>(),
                                k32.as<float>(), aniso ? kz32.as<float>() : nullptr, aniso, dmask.as<uint32_t>(),
                                (const float*)nullptr, partials.as<double>(), MODE_CG, ctl);
            ck(cudaEventRecord(ev3, stream), "event");
            ck(cudaEventSynchronize(ev3), "sync");
            float ms = 0.f;
            ck(cudaEventElapsedTime(&ms, ev2, ev3), "elapsed");
            if (r >= 0) total += ms;
        }
        ck(cudaGetLastError(), "launch");
        *avg_ms = total / reps;
        const double w = precision == 64 ? 8.0 : 4.0;
        // algorithmic bytes: read x, write y, one (isotropic) or two conductivity words per element
        *bytes = 2.0 * w * (double)N + 4.0 * (aniso ? 2.0 : 1.0) * (double)NE;
    }

    // y = A x with the system matrix of the current temperature (FemMatrix::mult, matrix.hpp:89):
    // after Dirichlet elimination, including the convective face terms.  Mesh-order arrays.
    // The FP32 operator exactly as one inner CG iteration applies it (the surface rows and
    // the stencil kernel the solve uses, with its (x, A x) partials reduced in a fixed order)
    // on a mesh-order vector; no Dirichlet replacement (the CG direction is zero on Dirichlet
    // nodes).  *staged: 1 when that kernel is the TMA-staged one.
    void cg_operator(const double* xin, double* yout, double* xax, int* staged) {
        check_device();
        if (!initialized) initialize();
        if (bc_dirty) materialize_bc();
        update_coef();
        DevBuf tmp, scratch;
        tmp.alloc((size_t)N * 8);
        scratch.alloc(sizeof(SolveCtl));
        SolveCtl* ctl = scratch.as<SolveCtl>();
        ck(cudaMemsetAsync(ctl, 0, sizeof(SolveCtl), stream), "memset");  // SOLVE_RUNNING
        ck(cudaMemcpyAsync(tmp.p, xin, (size_t)N * 8, cudaMemcpyHostToDevice, stream), "H2D x");
        launch_from_mesh_order_f64(cfg, n[0], n[1], n[2], n[0], n[1], n[2], ns[0], ns[1], ns[2], tmp.as<double>(),
                                   p64.as<double>(), 0.0);
        launch_norm2(cfg, N, p64.as<double>(), p32.as<float>(), partials.as<double>(), d_ctl.as<SolveCtl>(), 4);
        const bool fused = tma_ready();
        if (fused) {
            launch_operator_tma(cfg, tma, q32.as<float>(), partials.as<double>(), &ctl->status, ctl, tsurf);
            launch_partials_to_ctl(cfg, partials.as<double>(), tma_operator_blocks(tma), ctl);
        } else {
            op32(p32.as<float>(), q32.as<float>(), MODE_CG, ctl);
        }
        launch_widen(cfg, N, q32.as<float>(), q64.as<double>());
        launch_to_mesh_order_f64(cfg, n[0], n[1], n[2], n[0], (long long)n[0] * n[1], ns[0], ns[1], ns[2], 1,
                                 q64.as<double>(), tmp.as<double>());
        ck(cudaMemcpyAsync(yout, tmp.p, (size_t)N * 8, cudaMemcpyDeviceToHost, stream), "D2H y");
        ck(cudaMemcpyAsync(h_ctl, ctl, sizeof(SolveCtl), cudaMemcpyDeviceToHost, stream), "D2H ctl");
        ck(cudaStreamSynchronize(stream), "sync");
        if (xax) *xax = h_ctl->pq;
        if (staged) *staged = fused ? 1 : 0;
    }

    // the handle's buffers and stream belong to the device current at set-up
    void check_device() const {
        int dev = 0;
        ck(cudaGetDevice(&dev), "cudaGetDevice");
        if (dev != device)
            throw StateError("the current CUDA device (" + std::to_string(dev) + ") is not the device the handle "
                             "was created on (" + std::to_string(device) + ")");
    }

    void mult(int precision, const double* xin, double* yout) {
        check_device();
        if (!initialized) initialize();
        if (bc_dirty) materialize_bc();
        update_coef();
        DevBuf tmp;
        tmp.alloc((size_t)N * 8);
        ck(cudaMemcpyAsync(tmp.p, xin, (size_t)N * 8, cudaMemcpyHostToDevice, stream), "H2D x");
        launch_from_mesh_order_f64(cfg, n[0], n[1], n[2], n[0], n[1], n[2], ns[0], ns[1], ns[2], tmp.as<double>(),
                                   p64.as<double>(), 0.0);
        if (precision == 64) {
            op64(p64.as<double>(), q64.as<double>(), nullptr, MODE_MULT);
            launch_surface(cfg, s64, p64.as<double>(), q64.as<double>(), MODE_MULT);
        } else {
            launch_norm2(cfg, N, p64.as<double>(), p32.as<float>(), partials.as<double>(), d_ctl.as<SolveCtl>(), 4);
            op32(p32.as<float>(), q32.as<float>(), MODE_MULT);
            launch_surface(cfg, s32, p32.as<float>(), q32.as<float>(), MODE_MULT);
            launch_widen(cfg, N, q32.as<float>(), q64.as<double>());
        }
        launch_to_mesh_order_f64(cfg, n[0], n[1], n[2], n[0], (long long)n[0] * n[1], ns[0], ns[1], ns[2], 1,
                                 q64.as<double>(), tmp.as<double>());
        ck(cudaMemcpyAsync(yout, tmp.p, (size_t)N * 8, cudaMemcpyDeviceToHost, stream), "D2H y");
        ck(cudaStreamSynchronize(stream), "sync");
    }

    void mult_noalloc(int precision, const double* xin, double* yout);

    // ---------------------------------------------------------------------------------
    // outputs

    void get_temperature(double* out) {
        if (!initialized) {
            for (long long t = 0; t < n_active; ++t) out[t] = inittemp;
            return;
        }
        DevBuf tmp;
        if (masked) {
            tmp.alloc((size_t)n_active * 8);
            launch_gather(cfg, n_active, d_active.as<long long>(), T.as<double>(), tmp.as<double>());
        } else {
            tmp.alloc((size_t)N * 8);
            launch_to_mesh_order_f64(cfg, n[0], n[1], n[2], n[0], (long long)n[0] * n[1], ns[0], ns[1], ns[2], 1,
                                     T.as<double>(), tmp.as<double>());
        }
        ck(cudaMemcpyAsync(out, tmp.p, (size_t)n_active * 8, cudaMemcpyDeviceToHost, stream), "D2H T");
        ck(cudaStreamSynchronize(stream), "sync");
    }

    void set_temperature(const double* in) {
        if (!initialized) initialize();
        DevBuf tmp;
        tmp.alloc((size_t)n_active * 8);
        ck(cudaMemcpyAsync(tmp.p, in, (size_t)n_active * 8, cudaMemcpyHostToDevice, stream), "H2D T");
        if (masked)
            launch_scatter(cfg, n_active, d_active.as<long long>(), tmp.as<double>(), T.as<double>());
        else
            launch_from_mesh_order_f64(cfg, n[0], n[1], n[2], n[0], n[1], n[2], ns[0], ns[1], ns[2], tmp.as<double>(),
                                       T.as<double>(), 0.0);
        ck(cudaStreamSynchronize(stream), "sync");
    }

    void element_output(int comps, void (*fill)(plgpu_fem3d*, double*), double* out) {
        DevBuf canon, tmp;
        canon.alloc((size_t)NE * comps * 8);
        tmp.alloc((size_t)NE * comps * 8);
        fill(this, canon.as<double>());
        launch_to_mesh_order_f64(cfg, me(0), me(1), me(2), me(0), (long long)me(0) * me(1), es[0], es[1], es[2], comps,
                                 canon.as<double>(), tmp.as<double>());
        ck(cudaMemcpyAsync(out, tmp.p, (size_t)NE * comps * 8, cudaMemcpyDeviceToHost, stream), "D2H");
        ck(cudaStreamSynchronize(stream), "sync");
    }

    // 3 values per element (2 on a planar handle)
    void get_flux(double* out3) {
        if (!initialized) initialize();
        if (planar) {
            element_output(2,
                           [](plgpu_fem3d* h, double* dst) {
                               launch_flux2d(h->cfg, h->g64, h->T.as<double>(), h->d_mat.as<int>(),
                                             h->have_leaf ? h->d_hleaf.as<double>() : h->d_th.as<double>(), h->tab,
                                             dst);
                           },
                           out3);
            return;
        }
        element_output(3,
                       [](plgpu_fem3d* h, double* dst) {
                           launch_flux(h->cfg, h->g64, h->T.as<double>(), h->d_mat.as<int>(),
                                       h->have_leaf ? h->d_hleaf.as<double>() : h->d_th.as<double>(), h->tab, dst);
                       },
                       out3);
    }
    void get_conductivity(double* out2) {
        if (!initialized) initialize();
        element_output(2,
                       [](plgpu_fem3d* h, double* dst) {
                           if (h->planar)
                               launch_conductivity2d(h->cfg, h->n[0], h->n[1], h->T.as<double>(), h->d_mat.as<int>(),
                                                     h->d_th.as<double>(), h->tab, dst);
                           else
                               launch_conductivity(h->cfg, h->n[0], h->n[1], h->n[2], h->T.as<double>(),
                                                   h->d_mat.as<int>(), h->d_th.as<double>(), h->tab, dst);
                       },
                       out2);
    }
    void get_thickness(double* out) {
        if (!initialized) initialize();
        DevBuf tmp;
        tmp.alloc((size_t)NE * 8);
        launch_to_mesh_order_f64(cfg, me(0), me(1), me(2), n[0], (long long)n[0] * n[1], es[0], es[1], es[2], 1,
                                 d_th.as<double>(), tmp.as<double>());
        ck(cudaMemcpyAsync(out, tmp.p, (size_t)NE * 8, cudaMemcpyDeviceToHost, stream), "D2H");
        ck(cudaStreamSynchronize(stream), "sync");
    }
};

void plgpu_fem3d::mult_noalloc(int precision, const double* xin, double* yout) {
    if ((size_t)N > kNoAllocMaxNodes)
        throw ArgError("plgpu_fem3d_mult_noalloc handles meshes of at most " + std::to_string(kNoAllocMaxNodes) +
                       " nodes; this mesh has " + std::to_string(N) + " (use plgpu_fem3d_mult)");
    if (!initialized || bc_dirty)
        throw StateError("plgpu_fem3d_mult_noalloc needs a handle whose mesh, materials and boundary conditions "
                         "are already set up on the device: call plgpu_fem3d_compute or plgpu_fem3d_mult once first");
    check_device();
    double* stage = noalloc_stage(device);
    if (!stage)
        throw StateError("the no-allocation staging array has no device address on device " +
                         std::to_string(device));
    update_coef();
    ck(cudaMemcpyAsync(stage, xin, (size_t)N * 8, cudaMemcpyHostToDevice, stream), "H2D x");
    launch_from_mesh_order_f64(cfg, n[0], n[1], n[2], n[0], n[1], n[2], ns[0], ns[1], ns[2], stage, p64.as<double>(),
                               0.0);
    if (precision == 64) {
        op64(p64.as<double>(), q64.as<double>(), nullptr, MODE_MULT);
        launch_surface(cfg, s64, p64.as<double>(), q64.as<double>(), MODE_MULT);
    } else {
        launch_norm2(cfg, N, p64.as<double>(), p32.as<float>(), partials.as<double>(), d_ctl.as<SolveCtl>(), 4);
        op32(p32.as<float>(), q32.as<float>(), MODE_MULT);
        launch_surface(cfg, s32, p32.as<float>(), q32.as<float>(), MODE_MULT);
        launch_widen(cfg, N, q32.as<float>(), q64.as<double>());
    }
    launch_to_mesh_order_f64(cfg, n[0], n[1], n[2], n[0], (long long)n[0] * n[1], ns[0], ns[1], ns[2], 1,
                             q64.as<double>(), stage);
    ck(cudaMemcpyAsync(yout, stage, (size_t)N * 8, cudaMemcpyDeviceToHost, stream), "D2H y");
    ck(cudaStreamSynchronize(stream), "sync");
}

// ---------------------------------------------------------------------------------------
// Shockley3D (solvers/electrical/shockley/electr3d.cpp): the electrical solver runs on
// the thermal handle's mesh, operator, boundary elimination and linear solvers.  The
// potential lives in T, voltage conditions are the Dirichlet list, the load is zero
// and the conductivity tensor of every element is kept on the device (sig) between
// the junction updates.

struct plgpu_elec3d : plgpu_fem3d {
    std::vector<double> cxy, cz, epsr;
    std::vector<uint8_t> noheat;
    DevBuf d_cxy, d_cz, d_eps, d_noheat;
    std::vector<int32_t> host_junc;  // junction number + 1 per element, mesh order
    DevBuf d_junc;                   // same, padded canonical
    DevBuf d_over;                   // per-element (c00, c11) override, padded canonical
    bool have_over = false;
    DevBuf d_bj;                     // per-element (beta, js) override, padded canonical
    bool have_bj = false;
    std::vector<double> beta{std::nan("")}, js{1.0};  // BetaSolver(name), beta.cpp:18-22
    struct Region {
        int bottom = 0, top = 0;
        double height = 0.0;
        bool present = false;
    };
    std::vector<Region> regions;
    DevBuf d_info;
    DevBuf sig, jsave, cur, ebuf, wbuf;
    bool jsave_valid = false;
    double jc00 = 0.0, jc11 = 5.0;  // default junction conductivity (electr3d.hpp:143)
    int convergence = PLGPU_CONVERGENCE_FAST;
    bool have_potential = false;

    plgpu_elec3d() {
        inittemp = 0.0;  // potential.reset(size, 0.), electr3d.cpp:190
        maxerr = 0.05;   // [%], electr3d.cpp:27
        // conductivities span 1e-16..1e9 S/m (a junction between metal contacts): the
        // Jacobi-scaled residual converges the junction rows as tightly as the contacts
        plain_norm = false;
    }

    void setup(const double* a0, int n0, const double* a1, int n1, const double* a2, int n2, int ord) {
        setup_mesh(a0, n0, a1, n1, a2, n2, ord);
        aniso = true;  // c00 and c11 differ in junctions
        kz64.alloc((size_t)N * 8);
        kz32.alloc((size_t)N * 4);
        sig.alloc((size_t)N * 16);
        jsave.alloc((size_t)N * 16);
        cur.alloc((size_t)N * 24);
        ebuf.alloc((size_t)N * 24);
        wbuf.alloc((size_t)N * 8);
        d_junc.alloc((size_t)N * 4);
        ck(cudaMemsetAsync(d_junc.p, 0, (size_t)N * 4, stream), "memset");
        ck(cudaMemsetAsync(d_heat.p, 0, (size_t)N * 8, stream), "memset");
        ck(cudaStreamSynchronize(stream), "sync");
    }

    void set_materials_e(int nm, const double* c0, const double* c1, const double* ep, const uint8_t* em,
                         const uint8_t* nh) {
        if (nm <= 0 || !c0 || !c1) throw ArgError("material table needs cond_xy and cond_z");
        for (int m = 0; m < nm; ++m)
            if (!std::isfinite(c0[m]) || !std::isfinite(c1[m])) throw ArgError("conductivities must be finite");
        n_mat = nm;
        cxy.assign(c0, c0 + nm);
        cz.assign(c1, c1 + nm);
        epsr.assign(nm, 1.0);
        if (ep) epsr.assign(ep, ep + nm);
        empty.assign(nm, 0);
        if (em) empty.assign(em, em + nm);
        noheat.assign(nm, 0);
        if (nh) noheat.assign(nh, nh + nm);
        k300.assign(nm, 0.0);
        pexp.assign(nm, 0.0);
        kzr.assign(nm, 1.0);
        hexp.assign(nm, 0.0);
        upload(d_cxy, cxy, stream);
        upload(d_cz, cz, stream);
        upload(d_eps, epsr, stream);
        upload(d_noheat, noheat, stream);
        ck(cudaStreamSynchronize(stream), "sync");
        invalidate_graphs();
        invalidate_e();
    }

    void set_elements_e(const int32_t* mat, const int32_t* junc) {
        if (junc)
            for (long long e = 0; e < NE; ++e)
                if (junc[e] < 0) throw ArgError("junction numbers must be >= 0");
        set_elements(mat, nullptr, nullptr);
        host_junc.assign((size_t)NE, 0);
        if (junc) host_junc.assign(junc, junc + NE);
        DevBuf tmp;
        tmp.alloc((size_t)NE * 4);
        ck(cudaMemcpyAsync(tmp.p, host_junc.data(), (size_t)NE * 4, cudaMemcpyHostToDevice, stream), "H2D junc");
        launch_from_mesh_order_i32(cfg, n[0], n[1], n[2], n[0] - 1, n[1] - 1, n[2] - 1, es[0], es[1], es[2],
                                   tmp.as<int>(), d_junc.as<int>(), 0);
        ck(cudaStreamSynchronize(stream), "sync");
        invalidate_e();
    }

    // mesh-order (a, b) pairs per element -> padded canonical pairs in `dst` (zero padding)
    void upload_element_pairs(const double* src, DevBuf& dst) {
        dst.alloc((size_t)N * 16);
        DevBuf tmp;
        tmp.alloc((size_t)NE * 16);
        ck(cudaMemcpyAsync(tmp.p, src, (size_t)NE * 16, cudaMemcpyHostToDevice, stream), "H2D pairs");
        ck(cudaMemsetAsync(dst.p, 0, (size_t)N * 16, stream), "memset");
        std::vector<long long> idx((size_t)NE * 2);
        for (long long k = 0; k < n[2] - 1; ++k)
            for (long long j = 0; j < n[1] - 1; ++j)
                for (long long i = 0; i < n[0] - 1; ++i) {
                    const long long m = i * es[0] + j * es[1] + k * es[2];
                    const long long c = i + (long long)n[0] * (j + (long long)n[1] * k);
                    idx[(size_t)(2 * m)] = 2 * c;
                    idx[(size_t)(2 * m + 1)] = 2 * c + 1;
                }
        DevBuf d_idx;
        upload(d_idx, idx, stream);
        launch_scatter(cfg, NE * 2, d_idx.as<long long>(), tmp.as<double>(), dst.as<double>());
        ck(cudaStreamSynchronize(stream), "sync");
    }

    void set_override(const double* c2) {
        if (!have_elements) throw StateError("set the elements first");
        have_over = c2 != nullptr;
        if (c2)
            upload_element_pairs(c2, d_over);
        else
            d_over.release();
    }

    void set_junction_params(const double* bj) {
        if (!have_elements) throw StateError("set the elements first");
        have_bj = bj != nullptr;
        if (bj)
            upload_element_pairs(bj, d_bj);
        else
            d_bj.release();
    }

    void set_junction(int nj, double b, double j) {
        if (nj < 0) throw ArgError("junction number must be >= 0");
        if ((size_t)nj >= beta.size()) beta.resize((size_t)nj + 1, std::nan(""));
        if ((size_t)nj >= js.size()) js.resize((size_t)nj + 1, 1.0);
        beta[(size_t)nj] = b;
        js[(size_t)nj] = j;
        if (initialized) invalidate_e();  // setBeta / setJs invalidate the solver
    }

    void invalidate_e() {
        invalidate_solution();
        jsave_valid = false;
        have_potential = false;
    }

    // setupActiveRegions (electr3d.cpp:94-184): the node planes every junction spans
    void setup_regions() {
        int nreg = 0;
        for (int32_t v : host_junc) nreg = std::max(nreg, (int)v);
        regions.assign((size_t)nreg, Region{});
        for (int j = 0; j < n[1] - 1; ++j)
            for (int i = 0; i < n[0] - 1; ++i) {
                int num = 0, start = 0;
                for (int k = 0; k <= n[2] - 1; ++k) {
                    const int curr = k < n[2] - 1 ? host_junc[(size_t)(i * es[0] + j * es[1] + (long long)k * es[2])] : 0;
                    if (curr == num) continue;
                    if (num) {
                        Region& r = regions[(size_t)num - 1];
                        if (!r.present) {
                            r.present = true;
                            r.bottom = start;
                            r.top = k;
                        } else if (r.bottom != start || r.top != k) {
                            throw ArgError("Junction " + std::to_string(num - 1) +
                                           " does not have top and bottom edges at constant heights");
                        }
                    }
                    num = curr;
                    start = k;
                }
            }
        for (Region& r : regions)
            if (r.present) r.height = ax[2][(size_t)r.top] - ax[2][(size_t)r.bottom];
    }

    void upload_info() {
        std::vector<JunctionInfo> info(std::max<size_t>(regions.size(), 1));
        for (size_t r = 0; r < regions.size(); ++r) {
            if (!regions[r].present) continue;
            if (r >= beta.size()) throw StateError("no beta given for junction " + std::to_string(r));
            if (r >= js.size()) throw StateError("no js given for junction " + std::to_string(r));
            info[r] = JunctionInfo{regions[r].bottom, regions[r].top, regions[r].height, beta[r], js[r]};
        }
        upload(d_info, info, stream);
    }

    int active_regions() const {
        int c = 0;
        for (const Region& r : regions) c += r.present ? 1 : 0;
        return c;
    }

    void initialize_e() {
        initialize();
        setup_regions();
        upload_info();
        if (!jsave_valid) {
            launch_elec_fill_pairs(cfg, N, jsave.as<double>(), jc00, jc11);
            jsave_valid = true;
        }
        ck(cudaMemsetAsync(cur.p, 0, (size_t)N * 24, stream), "memset");
        ck(cudaStreamSynchronize(stream), "sync");
        have_potential = false;
    }

    void load_conductivity() {
        launch_elec_init_cond(cfg, n[0], n[1], n[2], d_mat.as<int>(), d_junc.as<int>(), d_info.as<JunctionInfo>(),
                              jsave.as<double>(), have_over ? d_over.as<double>() : nullptr, d_cxy.as<double>(),
                              d_cz.as<double>(), d_excl.as<uint8_t>(), sig.as<double>());
    }

    // ElectricalFem3DSolver::compute (electr3d.cpp:356-442)
    double compute_e(int loops, plgpu_stats* st) {
        NvtxRange nv("electrical compute");
        if (!initialized) initialize_e();
        if (bc_dirty) materialize_bc();
        upload_info();
        const long long launches0 = thread_launch_count();
        const int fallbacks0 = fallbacks;
        const long long learned0 = learned_iters;
        ck(cudaEventRecord(ev0, stream), "event");
        if (heat_dirty) build_static_load();  // zero load: no sources in the electrical problem
        log(3, "Running electrical calculations");
        load_conductivity();
        const int noactive = active_regions() == 0 ? 1 : 0;
        const double minj = 100e-7;  // no significant current below this [kA/cm2]
        const bool mixed = algorithm == PLGPU_ALGO_ITERATIVE || algorithm == PLGPU_ALGO_GPU_MIXED ||
                           algorithm == PLGPU_ALGO_GPU_LEARNED;
        double toterr = 0.0, err = 0.0, mcur = 0.0, relres = 0.0;
        int loop = 0, total_iters = 0, total_ref = 0;
        float solve_ms = 0.f;
        do {
            if (loopno != 0)
                launch_elec_junction_update(cfg, n[0], n[1], n[2], d_junc.as<int>(), d_info.as<JunctionInfo>(),
                                            have_bj ? d_bj.as<double>() : nullptr, T.as<double>(), convergence == PLGPU_CONVERGENCE_STABLE ? 1 : 0,
                                            sig.as<double>());
            launch_elec_coef(cfg, N, sig.as<double>(), k64.as<double>(), k32.as<float>(), kz64.as<double>(),
                             kz32.as<float>());
            refresh_tma();
            launch_diag(cfg, g64, k64.as<double>(), kz64.as<double>(), true, s64, dmask.as<uint32_t>(),
                        diag.as<double>(), minv64.as<double>(), minv32.as<float>());
            op64(vD.as<double>(), b.as<double>(), F.as<double>(), MODE_RHS);
            launch_set_dirichlet(cfg, (int)(d_didx.bytes / sizeof(int)), d_didx.as<int>(), d_dval.as<double>(),
                                 b.as<double>(), T.as<double>());
            ck(cudaGetLastError(), "launch");
            ck(cudaEventRecord(ev2, stream), "event");
            int status = 0, iters = 0, refs = 0;
            if (mixed)
                solve_mixed(status, iters, refs, relres);
            else
                solve_fp64(status, iters, relres);
            ck(cudaEventRecord(ev3, stream), "event");
            total_iters += iters;
            total_ref += refs;
            if (status == SOLVE_DEVICE_TIMEOUT)
                throw SolveError(PLGPU_ERR_CUDA, "a device-side wait for staged copies timed out");
            if (status == SOLVE_NONFINITE)
                throw SolveError(PLGPU_ERR_NONFINITE, "non-finite value in the linear solve");
            if (status == SOLVE_BREAKDOWN)
                throw SolveError(PLGPU_ERR_NOT_SPD, "stiffness matrix is not positive definite (CG breakdown)");
            converged = status == SOLVE_CONVERGED;
            if (!converged) {
                if (noconv == PLGPU_NOCONV_ERROR)
                    throw SolveError(PLGPU_ERR_NOCONV, "failed to converge in " + std::to_string(iters) +
                                                           " iterations (relative residual " +
                                                           std::to_string(relres) + ")");
                log(noconv == PLGPU_NOCONV_WARNING ? 2 : 5, "Failed to converge in %d iterations (error %g)", iters,
                    relres);
            }
            launch_elec_current(cfg, g64, T.as<double>(), sig.as<double>(), d_junc.as<int>(), d_mat.as<int>(),
                                d_excl.as<uint8_t>(), noactive, cur.as<double>(), partials.as<double>(),
                                d_ctl.as<SolveCtl>());
            SolveCtl c = read_ctl();
            float ms = 0.f;
            ck(cudaEventElapsedTime(&ms, ev2, ev3), "elapsed");
            solve_ms += ms;
            mcur = std::sqrt(c.red[1]);
            err = 100.0 * std::sqrt(c.red[0]) / std::max(mcur, minj);
            if ((loop != 0 || mcur >= minj) && err > toterr) toterr = err;
            ++loopno;
            ++loop;
            log(4, "Loop %d(%d): max(j%s) = %g kA/cm2, error = %g%%", loop, loopno, noactive ? "" : "@junc", mcur, err);
            if (loop >= kMaxOuterLoops) break;
        } while ((!converged || err > maxerr) && (loops == 0 || loop < loops));
        launch_elec_save_junction(cfg, n[0], n[1], n[2], d_junc.as<int>(), d_info.as<JunctionInfo>(),
                                  sig.as<double>(), jsave.as<double>());
        have_potential = true;
        ck(cudaEventRecord(ev1, stream), "event");
        ck(cudaEventSynchronize(ev1), "sync");
        float tot = 0.f;
        ck(cudaEventElapsedTime(&tot, ev0, ev1), "elapsed");
        if (st) {
            st->loops = loop;
            st->total_loops = loopno;
            st->inner_iterations = total_iters;
            st->refinements = total_ref;
            st->converged = converged ? 1 : 0;
            st->fallbacks = fallbacks - fallbacks0;
            st->learned_iterations = (int)(learned_iters - learned0);
            st->err = err;
            st->toterr = toterr;
            st->max_t = mcur;
            st->last_rel_residual = relres;
            st->solve_ms = solve_ms;
            st->total_ms = tot;
            st->kernel_launches = thread_launch_count() - launches0;
        }
        return toterr;
    }

    void need_potential(const char* what) const {
        if (!have_potential) throw StateError(std::string("no ") + what + ": run compute first");
    }

    // per-element field (comps per padded element) -> mesh order on the host
    void padded_elements_out(int comps, const double* padded, double* out) {
        DevBuf tmp;
        tmp.alloc((size_t)NE * comps * 8);
        launch_to_mesh_order_f64(cfg, n[0] - 1, n[1] - 1, n[2] - 1, n[0], (long long)n[0] * n[1], es[0], es[1], es[2],
                                 comps, padded, tmp.as<double>());
        ck(cudaMemcpyAsync(out, tmp.p, (size_t)NE * comps * 8, cudaMemcpyDeviceToHost, stream), "D2H");
        ck(cudaStreamSynchronize(stream), "sync");
    }

    void get_current(double* out3) {
        need_potential("current densities");
        launch_elec_masked_copy(cfg, n[0], n[1], n[2], 3, cur.as<double>(), d_mat.as<int>(), d_excl.as<uint8_t>(),
                                ebuf.as<double>());
        padded_elements_out(3, ebuf.as<double>(), out3);
    }

    void heat_padded(double* dst) {
        launch_elec_heat(cfg, g64, T.as<double>(), sig.as<double>(), d_mat.as<int>(), d_excl.as<uint8_t>(),
                         d_noheat.as<uint8_t>(), dst, 1);
    }

    void get_heat_e(double* out) {
        need_potential("heat densities");
        ck(cudaMemsetAsync(wbuf.p, 0, (size_t)N * 8, stream), "memset");
        heat_padded(wbuf.as<double>());
        padded_elements_out(1, wbuf.as<double>(), out);
    }

    // getConductivity (electr3d.cpp:557-565) reloads the conductivities first
    void get_conductivity_e(double* out2) {
        if (!initialized) initialize_e();
        upload_info();
        load_conductivity();
        launch_elec_masked_copy(cfg, n[0], n[1], n[2], 2, sig.as<double>(), d_mat.as<int>(), d_excl.as<uint8_t>(),
                                ebuf.as<double>());
        padded_elements_out(2, ebuf.as<double>(), out2);
    }

    double total_current(int nj) {
        need_potential("current densities");
        if (nj < 0 || (size_t)nj >= regions.size() || !regions[(size_t)nj].present)
            throw ArgError("wrong active region number");
        const Region& r = regions[(size_t)nj];
        launch_elec_plane_current(cfg, g64, cur.as<double>(), d_junc.as<int>(), (r.bottom + r.top) / 2,
                                  partials.as<double>(), d_ctl.as<SolveCtl>(), 6);
        return read_ctl().red[6] * 0.01;  // kA/cm2 um2 -> mA
    }

    double total_heat() {
        need_potential("heat densities");
        ck(cudaMemsetAsync(wbuf.p, 0, (size_t)N * 8, stream), "memset");
        heat_padded(wbuf.as<double>());
        launch_elec_volume_sum(cfg, g64, wbuf.as<double>(), d_mat.as<int>(), d_excl.as<uint8_t>(),
                               partials.as<double>(), d_ctl.as<SolveCtl>(), 5);
        return read_ctl().red[5] * 1e-15;  // um3 -> m3, W -> mW
    }

    double total_energy() {
        need_potential("potentials");
        launch_elec_energy_density(cfg, g64, T.as<double>(), d_mat.as<int>(), d_excl.as<uint8_t>(),
                                   d_eps.as<double>(), wbuf.as<double>());
        launch_elec_volume_sum(cfg, g64, wbuf.as<double>(), d_mat.as<int>(), d_excl.as<uint8_t>(),
                               partials.as<double>(), d_ctl.as<SolveCtl>(), 5);
        const double epsilon0 = 1.0 / (4e-7 * M_PI) / 299792458.0 / 299792458.0;  // plask/phys/constants.hpp:32-35
        return 0.5e-18 * epsilon0 * read_ctl().red[5];
    }

    double capacitance() {
        const auto& v = bcs[PLGPU_BC_TEMPERATURE];
        if (v.size() != 2)
            throw ArgError("cannot estimate applied voltage (exactly 2 voltage boundary conditions required)");
        const double U = v[0].v0 - v[1].v0;
        return 2e12 * total_energy() / (U * U);  // F -> pF
    }
};

// ---------------------------------------------------------------------------------------
// C ABI

namespace {
thread_local std::string g_create_error;

template <typename F>
int guarded(plgpu_fem3d* h, F&& f) {
    if (!h) return PLGPU_ERR_ARG;
    try {
        f();
        h->err.clear();
        return PLGPU_OK;
    } catch (const ArgError& e) {
        h->err = e.what();
        return PLGPU_ERR_ARG;
    } catch (const StateError& e) {
        h->err = e.what();
        return PLGPU_ERR_STATE;
    } catch (const SolveError& e) {
        h->err = e.what();
        return e.code;
    } catch (const CudaError& e) {
        h->err = e.what();
        return PLGPU_ERR_CUDA;
    } catch (const std::exception& e) {
        h->err = e.what();
        return PLGPU_ERR_ARG;
    }
}
}  // namespace

namespace {
template <typename F>
int guarded_net(plgpu_unet* net, F&& f) {
    if (!net) return PLGPU_ERR_ARG;
    try {
        f();
        net->err.clear();
        return PLGPU_OK;
    } catch (const ArgError& e) {
        net->err = e.what();
        return PLGPU_ERR_ARG;
    } catch (const std::exception& e) {
        net->err = e.what();
        return PLGPU_ERR_CUDA;
    }
}
constexpr char kNetMagic[8] = {'P', 'L', 'G', 'P', 'U', 'N', 'E', 'T'};
constexpr uint32_t kNetVersion = 1;
}  // namespace

extern "C" {

int plgpu_fem3d_create(const double* ax0, int n0, const double* ax1, int n1, const double* ax2, int n2, int ordering,
                       plgpu_fem3d** out) {
    if (!out) return PLGPU_ERR_ARG;
    *out = nullptr;
    std::unique_ptr<plgpu_fem3d> h(new plgpu_fem3d());
    try {
        h->setup_mesh(ax0, n0, ax1, n1, ax2, n2, ordering);
    } catch (const ArgError& e) {
        g_create_error = e.what();
        return PLGPU_ERR_ARG;
    } catch (const std::exception& e) {
        g_create_error = e.what();
        return PLGPU_ERR_CUDA;
    }
    *out = h.release();
    return PLGPU_OK;
}

int plgpu_fem2d_create(const double* ax0, int n0, const double* ax1, int n1, int ordering, int geometry,
                       plgpu_fem3d** out) {
    if (!out) return PLGPU_ERR_ARG;
    *out = nullptr;
    if (ordering != PLGPU_ORDER2D_10 && ordering != PLGPU_ORDER2D_01) {
        g_create_error = "unknown 2D iteration order";
        return PLGPU_ERR_ARG;
    }
    if (geometry != PLGPU_GEOMETRY_CARTESIAN && geometry != PLGPU_GEOMETRY_CYLINDRICAL) {
        g_create_error = "unknown 2D geometry";
        return PLGPU_ERR_ARG;
    }
    std::unique_ptr<plgpu_fem3d> h(new plgpu_fem3d());
    try {
        // the node plane is the major (outermost) axis 2 of size 1: ORDER_10 (axis 0
        // fastest) is the 3D order 210, ORDER_01 (axis 1 fastest) the order 201
        const double z0 = 0.0;
        h->setup_mesh(ax0, n0, ax1, n1, &z0, 1, ordering == PLGPU_ORDER2D_10 ? PLGPU_ORDER_210 : PLGPU_ORDER_201,
                      geometry);
    } catch (const ArgError& e) {
        g_create_error = e.what();
        return PLGPU_ERR_ARG;
    } catch (const std::exception& e) {
        g_create_error = e.what();
        return PLGPU_ERR_CUDA;
    }
    *out = h.release();
    return PLGPU_OK;
}

int plgpu_fem3d_destroy(plgpu_fem3d* h) {
    if (!h) return PLGPU_ERR_ARG;
    if (h->stream) cudaStreamSynchronize(h->stream);
    delete h;
    return PLGPU_OK;
}

const char* plgpu_fem3d_last_error(const plgpu_fem3d* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

int plgpu_fem3d_set_materials(plgpu_fem3d* h, int n_mat, const double* k300, const double* p, const double* kz_ratio,
                              const double* hexp, const uint8_t* empty) {
    return guarded(h, [&] { h->set_materials(n_mat, k300, p, kz_ratio, hexp, empty); });
}

int plgpu_fem3d_set_material_table(plgpu_fem3d* h, int material, int n_points, const double* T, const double* k_xy,
                                   const double* k_z) {
    return guarded(h, [&] { h->set_material_table(material, n_points, T, k_xy, k_z); });
}

int plgpu_fem3d_set_elements(plgpu_fem3d* h, const int32_t* material, const double* heat, const double* leaf_height) {
    return guarded(h, [&] { h->set_elements(material, heat, leaf_height); });
}

int plgpu_fem3d_set_heat(plgpu_fem3d* h, const double* heat) {
    return guarded(h, [&] { h->set_heat(heat); });
}

int plgpu_fem3d_clear_bc(plgpu_fem3d* h, int kind) {
    return guarded(h, [&] {
        if (kind < 0 || kind > 3) throw ArgError("unknown boundary-condition kind");
        h->bcs[kind].clear();
        h->bc_dirty = true;
    });
}

int plgpu_fem3d_add_bc(plgpu_fem3d* h, int kind, const int64_t* nodes, size_t count, double v0, double v1) {
    return guarded(h, [&] {
        if (kind < 0 || kind > 3) throw ArgError("unknown boundary-condition kind");
        if (count && !nodes) throw ArgError("null node list");
        plgpu_fem3d::Cond c;
        c.nodes.assign(nodes, nodes + count);
        for (int64_t m : c.nodes)
            if (m < 0 || m >= h->N) throw ArgError("boundary node index out of range");
        c.v0 = v0;
        c.v1 = v1;
        h->bcs[kind].push_back(std::move(c));
        h->bc_dirty = true;
    });
}

int plgpu_fem3d_set_solver(plgpu_fem3d* h, int algorithm, double rtol, int maxit, int noconv, int empty_elements,
                           int bc_compat) {
    return guarded(h, [&] {
        if (algorithm < 0 || algorithm > PLGPU_ALGO_GPU_LEARNED) throw ArgError("unknown algorithm");
        if (!(rtol > 0.0) || rtol >= 1.0) throw ArgError("rtol must be in (0, 1)");
        if (noconv < 0 || noconv > 2) throw ArgError("unknown noconv behaviour");
        if (empty_elements < 0 || empty_elements > 2) throw ArgError("unknown empty-elements mode");
        const bool remask = h->exclude_empty();
        h->algorithm = algorithm;
        h->rtol = rtol;
        h->maxit = maxit;
        h->noconv = noconv;
        h->empty_mode = empty_elements;
        if (h->bc_compat != (bc_compat ? 1 : 0)) h->bc_dirty = true;
        h->bc_compat = bc_compat ? 1 : 0;
        if (remask != h->exclude_empty()) h->invalidate_solution();
    });
}

int plgpu_fem3d_set_residual_norm(plgpu_fem3d* h, int norm) {
    return guarded(h, [&] {
        if (norm != PLGPU_NORM_SCALED && norm != PLGPU_NORM_PLAIN) throw ArgError("unknown residual norm");
        h->plain_norm = norm == PLGPU_NORM_PLAIN;
    });
}

int plgpu_fem3d_set_loop(plgpu_fem3d* h, double inittemp, double maxerr) {
    return guarded(h, [&] {
        if (!std::isfinite(inittemp) || !(maxerr >= 0.0)) throw ArgError("bad inittemp or maxerr");
        h->inittemp = inittemp;
        h->maxerr = maxerr;
    });
}

int plgpu_fem3d_compute(plgpu_fem3d* h, int loops, double* toterr, plgpu_stats* stats) {
    return guarded(h, [&] {
        if (loops < 0) throw ArgError("loops must be >= 0");
        const double t = h->compute(loops, stats);
        if (toterr) *toterr = t;
    });
}

int plgpu_fem3d_invalidate(plgpu_fem3d* h) {
    return guarded(h, [&] { h->invalidate_solution(); });
}

int plgpu_fem3d_sizes(const plgpu_fem3d* h, size_t* n_nodes, size_t* n_elements) {
    if (!h) return PLGPU_ERR_ARG;
    plgpu_fem3d* m = const_cast<plgpu_fem3d*>(h);
    return guarded(m, [&] {
        if (!m->initialized && m->have_elements && m->n_mat) m->initialize();
        if (n_nodes) *n_nodes = (size_t)(m->initialized ? m->n_active : m->N);
        if (n_elements) *n_elements = (size_t)m->NE;
    });
}

int plgpu_fem3d_get_temperature(plgpu_fem3d* h, double* out) {
    return guarded(h, [&] {
        if (!out) throw ArgError("null output");
        h->get_temperature(out);
    });
}

int plgpu_fem3d_set_temperature(plgpu_fem3d* h, const double* in) {
    return guarded(h, [&] {
        if (!in) throw ArgError("null input");
        h->set_temperature(in);
    });
}

int plgpu_fem3d_get_heat_flux(plgpu_fem3d* h, double* out3) {
    return guarded(h, [&] {
        if (!out3) throw ArgError("null output");
        h->get_flux(out3);
    });
}

int plgpu_fem3d_get_conductivity(plgpu_fem3d* h, double* out2) {
    return guarded(h, [&] {
        if (!out2) throw ArgError("null output");
        h->get_conductivity(out2);
    });
}

int plgpu_fem3d_get_thickness(plgpu_fem3d* h, double* out) {
    return guarded(h, [&] {
        if (!out) throw ArgError("null output");
        h->get_thickness(out);
    });
}

void* plgpu_fem3d_stream(plgpu_fem3d* h) { return h ? (void*)h->stream : nullptr; }

int plgpu_fem3d_mult(plgpu_fem3d* h, int precision, const double* x, double* y) {
    return guarded(h, [&] {
        if (precision != 32 && precision != 64) throw ArgError("precision must be 32 or 64");
        if (!x || !y) throw ArgError("null vector");
        h->mult(precision, x, y);
    });
}

int plgpu_fem3d_mult_noalloc(plgpu_fem3d* h, int precision, const double* x, double* y) {
    return guarded(h, [&] {
        if (precision != 32 && precision != 64) throw ArgError("precision must be 32 or 64");
        if (!x || !y) throw ArgError("null vector");
        h->mult_noalloc(precision, x, y);
    });
}

int plgpu_fem3d_cg_operator(plgpu_fem3d* h, const double* x, double* y, double* xax, int* staged) {
    return guarded(h, [&] {
        if (!x || !y) throw ArgError("null vector");
        h->cg_operator(x, y, xax, staged);
    });
}

int plgpu_fem3d_time_operator(plgpu_fem3d* h, int precision, int reps, int flush_l2, double* avg_ms,
                              double* bytes_per_launch) {
    return guarded(h, [&] {
        if (precision != 32 && precision != 64) throw ArgError("precision must be 32 or 64");
        if (!avg_ms || !bytes_per_launch) throw ArgError("null output");
        h->time_operator(precision, reps, flush_l2, avg_ms, bytes_per_launch);
    });
}

// ---------------------------------------------------------------------------------------
// learned preconditioner (include/plgpu_unet.h)


int plgpu_unet_create(unsigned long long seed, plgpu_unet** out) {
    if (!out) return PLGPU_ERR_ARG;
    *out = nullptr;
    std::unique_ptr<plgpu_unet> net(new plgpu_unet());
    try {
        net->model.allocate();
        net->model.init(seed);
    } catch (const std::exception& e) {
        g_create_error = e.what();
        return PLGPU_ERR_CUDA;
    }
    *out = net.release();
    return PLGPU_OK;
}

int plgpu_unet_destroy(plgpu_unet* net) {
    if (!net) return PLGPU_ERR_ARG;
    cudaDeviceSynchronize();
    delete net;
    return PLGPU_OK;
}

const char* plgpu_unet_last_error(const plgpu_unet* net) { return net ? net->err.c_str() : g_create_error.c_str(); }

int plgpu_unet_num_params(const plgpu_unet* net, size_t* n) {
    if (!net || !n) return PLGPU_ERR_ARG;
    *n = net->model.n_params;
    return PLGPU_OK;
}

int plgpu_unet_get_weights(plgpu_unet* net, float* out) {
    return guarded_net(net, [&] {
        if (!out) throw ArgError("null output");
        cudaDeviceSynchronize();
        net->model.download(out);
    });
}

int plgpu_unet_set_weights(plgpu_unet* net, const float* in) {
    return guarded_net(net, [&] {
        if (!in) throw ArgError("null input");
        cudaDeviceSynchronize();
        net->model.upload(in);
    });
}

int plgpu_unet_save(plgpu_unet* net, const char* path) {
    return guarded_net(net, [&] {
        if (!path) throw ArgError("null path");
        std::vector<float> w(net->model.n_params);
        cudaDeviceSynchronize();
        net->model.download(w.data());
        const uint64_t n = w.size(), sum = unet_checksum(w.data(), w.size());
        std::ofstream f(path, std::ios::binary);
        if (!f) throw ArgError(std::string("cannot write ") + path);
        f.write(kNetMagic, 8);
        f.write(reinterpret_cast<const char*>(&kNetVersion), 4);
        f.write(reinterpret_cast<const char*>(&n), 8);
        f.write(reinterpret_cast<const char*>(w.data()), (std::streamsize)(n * 4));
        f.write(reinterpret_cast<const char*>(&sum), 8);
        if (!f) throw ArgError(std::string("write failed: ") + path);
    });
}

int plgpu_unet_load(plgpu_unet* net, const char* path) {
    return guarded_net(net, [&] {
        if (!path) throw ArgError("null path");
        std::ifstream f(path, std::ios::binary);
        if (!f) throw ArgError(std::string("cannot read ") + path);
        char magic[8];
        uint32_t ver = 0;
        uint64_t n = 0, sum = 0;
        f.read(magic, 8);
        f.read(reinterpret_cast<char*>(&ver), 4);
        f.read(reinterpret_cast<char*>(&n), 8);
        if (!f || std::memcmp(magic, kNetMagic, 8) != 0) throw ArgError("not a network weights file");
        if (ver != kNetVersion) throw ArgError("unsupported weights file version");
        if (n != net->model.n_params) throw ArgError("weights file does not match the network architecture");
        std::vector<float> w(n);
        f.read(reinterpret_cast<char*>(w.data()), (std::streamsize)(n * 4));
        f.read(reinterpret_cast<char*>(&sum), 8);
        if (!f) throw ArgError("truncated weights file");
        if (sum != unet_checksum(w.data(), w.size())) throw ArgError("weights file checksum mismatch");
        cudaDeviceSynchronize();
        net->model.upload(w.data());
    });
}

int plgpu_unet_train(plgpu_unet* net, plgpu_fem3d* fem, int steps, float lr, unsigned long long seed, int smooth_min,
                     int smooth_max, int pair_kind, float* losses) {
    if (!net) return PLGPU_ERR_ARG;
    return guarded(fem, [&] {
        if (fem->planar) throw ArgError("the learned preconditioner is 3D only");
        fem->train(net, steps, lr, seed, smooth_min, smooth_max, pair_kind, losses);
    });
}

int plgpu_unet_loss_grad(plgpu_unet* net, plgpu_fem3d* fem, const double* e, double* loss, float* grad, double* r_out,
                         double* z_out) {
    if (!net) return PLGPU_ERR_ARG;
    return guarded(fem, [&] {
        if (!e || !loss || !grad) throw ArgError("null argument");
        if (fem->planar) throw ArgError("the learned preconditioner is 3D only");
        fem->loss_grad(net, e, loss, grad, r_out, z_out);
    });
}

int plgpu_unet_apply(plgpu_unet* net, plgpu_fem3d* fem, const double* r, double* z) {
    if (!net) return PLGPU_ERR_ARG;
    return guarded(fem, [&] {
        if (!r || !z) throw ArgError("null argument");
        if (fem->planar) throw ArgError("the learned preconditioner is 3D only");
        fem->apply_net(net, r, z);
    });
}

int plgpu_unet_time_apply(plgpu_unet* net, plgpu_fem3d* fem, int reps, double* forward_ms, double* apply_ms) {
    if (!net) return PLGPU_ERR_ARG;
    return guarded(fem, [&] {
        if (!forward_ms || !apply_ms) throw ArgError("null argument");
        if (fem->planar) throw ArgError("the learned preconditioner is 3D only");
        fem->time_net(net, reps, forward_ms, apply_ms);
    });
}

int plgpu_fem3d_set_preconditioner(plgpu_fem3d* fem, plgpu_unet* net) {
    return guarded(fem, [&] {
        if (fem->planar && net) throw ArgError("the learned preconditioner is 3D only");
        fem->pre = net;
        fem->invalidate_graphs();
    });
}

int plgpu_fem3d_set_log_callback(plgpu_fem3d* h, void (*cb)(void*, int, const char*), void* user) {
    return guarded(h, [&] {
        h->log_cb = cb;
        h->log_user = user;
    });
}

// ---------------------------------------------------------------------------------------
// Shockley3D

int plgpu_elec3d_create(const double* ax0, int n0, const double* ax1, int n1, const double* ax2, int n2, int ordering,
                        plgpu_elec3d** out) {
    if (!out) return PLGPU_ERR_ARG;
    *out = nullptr;
    std::unique_ptr<plgpu_elec3d> h(new plgpu_elec3d());
    try {
        h->setup(ax0, n0, ax1, n1, ax2, n2, ordering);
    } catch (const ArgError& e) {
        g_create_error = e.what();
        return PLGPU_ERR_ARG;
    } catch (const std::exception& e) {
        g_create_error = e.what();
        return PLGPU_ERR_CUDA;
    }
    *out = h.release();
    return PLGPU_OK;
}

int plgpu_elec3d_destroy(plgpu_elec3d* h) {
    if (!h) return PLGPU_ERR_ARG;
    delete h;
    return PLGPU_OK;
}

const char* plgpu_elec3d_last_error(const plgpu_elec3d* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

int plgpu_elec3d_set_materials(plgpu_elec3d* h, int n_mat, const double* cond_xy, const double* cond_z,
                               const double* eps, const uint8_t* empty, const uint8_t* noheat) {
    return guarded(h, [&] { h->set_materials_e(n_mat, cond_xy, cond_z, eps, empty, noheat); });
}

int plgpu_elec3d_set_elements(plgpu_elec3d* h, const int32_t* material, const int32_t* junction) {
    return guarded(h, [&] { h->set_elements_e(material, junction); });
}

int plgpu_elec3d_set_element_conductivity(plgpu_elec3d* h, const double* cond2) {
    return guarded(h, [&] { h->set_override(cond2); });
}

int plgpu_elec3d_set_junction_params(plgpu_elec3d* h, const double* beta_js) {
    return guarded(h, [&] { h->set_junction_params(beta_js); });
}

int plgpu_elec3d_set_junction(plgpu_elec3d* h, int n, double beta, double js) {
    return guarded(h, [&] { h->set_junction(n, beta, js); });
}

int plgpu_elec3d_set_junction_conductivity(plgpu_elec3d* h, double c00, double c11) {
    return guarded(h, [&] {
        if (!std::isfinite(c00) || !std::isfinite(c11)) throw ArgError("junction conductivity must be finite");
        h->jc00 = c00;
        h->jc11 = c11;
        h->jsave_valid = false;
        if (h->initialized) {
            launch_elec_fill_pairs(h->cfg, h->N, h->jsave.as<double>(), c00, c11);
            ck(cudaStreamSynchronize(h->stream), "sync");
            h->jsave_valid = true;
        }
    });
}

int plgpu_elec3d_clear_voltage(plgpu_elec3d* h) {
    return guarded(h, [&] {
        h->bcs[PLGPU_BC_TEMPERATURE].clear();
        h->bc_dirty = true;
    });
}

int plgpu_elec3d_add_voltage(plgpu_elec3d* h, const int64_t* nodes, size_t count, double volts) {
    return guarded(h, [&] {
        if (count && !nodes) throw ArgError("null node list");
        if (!std::isfinite(volts)) throw ArgError("voltage must be finite");
        for (size_t t = 0; t < count; ++t)
            if (nodes[t] < 0 || nodes[t] >= h->N) throw ArgError("boundary node index out of range");
        plgpu_fem3d::Cond c;
        c.nodes.assign(nodes, nodes + count);
        c.v0 = volts;
        c.v1 = 0.0;
        h->bcs[PLGPU_BC_TEMPERATURE].push_back(std::move(c));
        h->bc_dirty = true;
    });
}

int plgpu_elec3d_set_solver(plgpu_elec3d* h, int algorithm, double rtol, int maxit, int noconv, int empty_elements) {
    return plgpu_fem3d_set_solver(h, algorithm, rtol, maxit, noconv, empty_elements, 1);
}

int plgpu_elec3d_set_loop(plgpu_elec3d* h, double maxerr, int convergence) {
    return guarded(h, [&] {
        if (!(maxerr >= 0.0)) throw ArgError("maxerr must be >= 0");
        if (convergence != PLGPU_CONVERGENCE_FAST && convergence != PLGPU_CONVERGENCE_STABLE)
            throw ArgError("unknown convergence mode");
        h->maxerr = maxerr;
        h->convergence = convergence;
    });
}

int plgpu_elec3d_compute(plgpu_elec3d* h, int loops, double* toterr, plgpu_stats* stats) {
    return guarded(h, [&] {
        if (loops < 0) throw ArgError("loops must be >= 0");
        const double t = h->compute_e(loops, stats);
        if (toterr) *toterr = t;
    });
}

int plgpu_elec3d_invalidate(plgpu_elec3d* h) {
    return guarded(h, [&] { h->invalidate_e(); });
}

int plgpu_elec3d_get_potential(plgpu_elec3d* h, double* out) {
    return guarded(h, [&] {
        if (!out) throw ArgError("null output");
        h->need_potential("potentials");
        h->get_temperature(out);
    });
}

int plgpu_elec3d_get_current_density(plgpu_elec3d* h, double* out3) {
    return guarded(h, [&] {
        if (!out3) throw ArgError("null output");
        h->get_current(out3);
    });
}

int plgpu_elec3d_get_heat(plgpu_elec3d* h, double* out) {
    return guarded(h, [&] {
        if (!out) throw ArgError("null output");
        h->get_heat_e(out);
    });
}

int plgpu_elec3d_get_conductivity(plgpu_elec3d* h, double* out2) {
    return guarded(h, [&] {
        if (!out2) throw ArgError("null output");
        h->get_conductivity_e(out2);
    });
}

int plgpu_elec3d_total_current(plgpu_elec3d* h, int n, double* mA) {
    return guarded(h, [&] {
        if (!mA) throw ArgError("null output");
        *mA = h->total_current(n);
    });
}

int plgpu_elec3d_total_heat(plgpu_elec3d* h, double* mW) {
    return guarded(h, [&] {
        if (!mW) throw ArgError("null output");
        *mW = h->total_heat();
    });
}

int plgpu_elec3d_total_energy(plgpu_elec3d* h, double* J) {
    return guarded(h, [&] {
        if (!J) throw ArgError("null output");
        *J = h->total_energy();
    });
}

int plgpu_elec3d_capacitance(plgpu_elec3d* h, double* pF) {
    return guarded(h, [&] {
        if (!pF) throw ArgError("null output");
        *pF = h->capacitance();
    });
}

void* plgpu_elec3d_stream(plgpu_elec3d* h) { return h ? (void*)h->stream : nullptr; }

int plgpu_fem3d_heat_from(plgpu_fem3d* thermal, plgpu_elec3d* electrical) {
    if (!electrical) return PLGPU_ERR_ARG;
    return guarded(thermal, [&] {
        if (thermal == electrical) throw ArgError("the thermal and electrical handles must differ");
        if (thermal->planar) throw ArgError("a 2D thermal handle cannot take 3D heat");
        for (int d = 0; d < 3; ++d)
            if (thermal->ax[d] != electrical->ax[d])
                throw ArgError("thermal and electrical meshes differ (interpolate on the host instead)");
        electrical->need_potential("heat densities");
        electrical->heat_padded(thermal->d_heat.as<double>());
        ck(cudaStreamSynchronize(electrical->stream), "sync");
        thermal->heat_dirty = true;
    });
}

int plgpu_fem3d_get_element_temperature(plgpu_fem3d* h, double* out) {
    return guarded(h, [&] {
        if (!out) throw ArgError("null output");
        if (h->planar) throw ArgError("element temperatures are provided for 3D handles");
        if (!h->initialized) {
            for (long long e = 0; e < h->NE; ++e) out[e] = h->inittemp;
            return;
        }
        DevBuf avg, tmp;
        avg.alloc((size_t)h->N * 8);
        tmp.alloc((size_t)h->NE * 8);
        launch_elem_average(h->cfg, h->n[0], h->n[1], h->n[2], h->T.as<double>(), avg.as<double>());
        launch_to_mesh_order_f64(h->cfg, h->n[0] - 1, h->n[1] - 1, h->n[2] - 1, h->n[0], (long long)h->n[0] * h->n[1],
                                 h->es[0], h->es[1], h->es[2], 1, avg.as<double>(), tmp.as<double>());
        ck(cudaMemcpyAsync(out, tmp.p, (size_t)h->NE * 8, cudaMemcpyDeviceToHost, h->stream), "D2H");
        ck(cudaStreamSynchronize(h->stream), "sync");
    });
}


// ---------------------------------------------------------------------------------------
// Batched solves: independent handles computed concurrently, each from its own host
// thread on its own stream, so that the kernels of different solves share the SMs.

int plgpu_fem3d_set_grid_share(plgpu_fem3d* h, int share) {
    return guarded(h, [&] {
        if (share < 1) throw ArgError("grid share must be >= 1");
        if (h->cfg.op_share != share) {
            h->cfg.op_share = share;
            h->invalidate_graphs();  // captured launches carry the old grid
        }
    });
}

int plgpu_fem3d_batch_compute(plgpu_fem3d* const* handles, int count, int loops, int threads, double* toterr,
                              plgpu_stats* stats, int* status) {
    if (!handles || count < 0 || loops < 0) return PLGPU_ERR_ARG;
    for (int i = 0; i < count; ++i) {
        if (!handles[i]) return PLGPU_ERR_ARG;
        for (int j = 0; j < i; ++j)
            if (handles[j] == handles[i]) return PLGPU_ERR_ARG;  // one host thread per handle
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return PLGPU_ERR_CUDA;
    std::atomic<int> next{0};
    std::vector<int> st((size_t)count, PLGPU_OK);
    auto worker = [&]() {
        cudaSetDevice(dev);
        for (;;) {
            const int i = next.fetch_add(1);
            if (i >= count) break;
            plgpu_fem3d* h = handles[i];
            st[(size_t)i] = guarded(h, [&] {
                const double t = h->compute(loops, stats ? &stats[i] : nullptr);
                if (toterr) toterr[i] = t;
            });
        }
    };
    const int nt = std::max(1, std::min(threads, std::max(count, 1)));
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; ++t) pool.emplace_back(worker);
    worker();
    for (auto& th : pool) th.join();
    int rc = PLGPU_OK;
    for (int i = 0; i < count; ++i) {
        if (status) status[i] = st[(size_t)i];
        if (rc == PLGPU_OK && st[(size_t)i] != PLGPU_OK) rc = st[(size_t)i];
    }
    return rc;
}

int plgpu_fem3d_batch_tune(plgpu_fem3d* const* handles, int count, int loops, int max_threads, int* best_threads,
                           int* best_share, double* timings) {
    if (!handles || count <= 0 || max_threads < 1) return PLGPU_ERR_ARG;
    double best = -1.0;
    int bt = 1, bs = 1, trial = 0;
    for (int t = 1; t <= std::min(max_threads, count); t *= 2) {
        for (int policy = 0; policy < 2; ++policy) {
            const int share = policy == 0 ? 1 : t;
            if (policy == 1 && t == 1) {  // same as the whole-GPU grid
                if (timings) timings[trial] = timings[trial - 1];
                ++trial;
                continue;
            }
            for (int i = 0; i < count; ++i) {
                int rc = plgpu_fem3d_set_grid_share(handles[i], share);
                if (rc == PLGPU_OK) rc = plgpu_fem3d_invalidate(handles[i]);
                if (rc != PLGPU_OK) return rc;
            }
            if (cudaDeviceSynchronize() != cudaSuccess) return PLGPU_ERR_CUDA;
            const auto t0 = std::chrono::steady_clock::now();
            const int rc = plgpu_fem3d_batch_compute(handles, count, loops, t, nullptr, nullptr, nullptr);
            if (rc != PLGPU_OK) return rc;
            const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            const double rate = sec > 0 ? count / sec : 0.0;
            if (timings) timings[trial] = rate;
            ++trial;
            if (rate > best) {
                best = rate;
                bt = t;
                bs = share;
            }
        }
    }
    for (int i = 0; i < count; ++i) {
        const int rc = plgpu_fem3d_set_grid_share(handles[i], bs);
        if (rc != PLGPU_OK) return rc;
    }
    if (best_threads) *best_threads = bt;
    if (best_share) *best_share = bs;
    return PLGPU_OK;
}


// ---------------------------------------------------------------------------------------
// Time stepping

int plgpu_fem3d_set_dynamic(plgpu_fem3d* h, const double* cp, const double* dens, double timestep,
                            double methodparam, int lumping, int rebuildfreq, int logfreq) {
    return guarded(h, [&] {
        if (h->n_mat == 0) throw StateError("set the material table first");
        if (!cp || !dens) throw ArgError("cp and dens are required");
        if (!(timestep > 0.0) || !std::isfinite(timestep)) throw ArgError("timestep must be positive");
        if (!(methodparam >= 0.0 && methodparam <= 1.0)) throw ArgError("methodparam must be in [0, 1]");
        if (rebuildfreq < 0 || logfreq < 0) throw ArgError("frequencies must be >= 0");
        for (int m = 0; m < h->n_mat; ++m)
            if (!std::isfinite(cp[m]) || !std::isfinite(dens[m]) || cp[m] < 0 || dens[m] < 0)
                throw ArgError("cp and dens must be finite and >= 0");
        h->cp_tab.assign(cp, cp + h->n_mat);
        h->dens_tab.assign(dens, dens + h->n_mat);
        h->dyn_dt = timestep;
        h->dyn_theta = methodparam;
        h->dyn_lumping = lumping != 0;
        h->dyn_rebuild = rebuildfreq;
        h->dyn_logfreq = logfreq;
    });
}

int plgpu_fem3d_compute_dynamic(plgpu_fem3d* h, double time, double* elapsed, plgpu_stats* stats) {
    return guarded(h, [&] {
        if (!std::isfinite(time) || time < 0.0) throw ArgError("time must be finite and >= 0");
        h->compute_dynamic(time, stats);
        if (elapsed) *elapsed = h->elapstime;
    });
}

}  // extern "C"
