// smip_api.cu -- host runtime behind the C ABI (include/smip_gpu.h).
//
// A stack owns the device-resident accumulators of one speckle-masking job
// and runs the per-frame pipeline in batches on its CUDA stream:
//
//   raw frames -> row FFT -> column FFT (S, |F|^2, correlation columns)
//              -> correlation rows -> integer shifts -> shift-and-add
//              -> bispectrum accumulation over the whole batch
//
// Only the final reconstruction steps (phase recovery, image) and result
// downloads synchronise the stream.  The spiral visit list of
// NextRecoIndex is host arithmetic (phasereco.cpp:17-36), computed once per
// radius and uploaded.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/smip_gpu.h"
#include "smip_internal.h"

using namespace smip_gpu;

// ------------------------------------------------------------------ errors
static thread_local std::string g_last_error;

static int fail(int code, const std::string& msg)
{
    g_last_error = msg;
    return code;
}

#define CUDA_TRY(expr)                                                                                     \
    do {                                                                                                   \
        cudaError_t e_ = (expr);                                                                           \
        if (e_ != cudaSuccess)                                                                             \
            return fail(e_ == cudaErrorMemoryAllocation ? SMIP_E_NO_MEMORY : SMIP_E_CUDA,                  \
                        std::string(#expr) + ": " + cudaGetErrorString(e_));                               \
    } while (0)

extern "C" const char* smip_last_error(void) { return g_last_error.c_str(); }

void smip_gpu::set_error_message(const std::string& m) { g_last_error = m; }

static std::atomic<long long> g_launches { 0 };
void smip_gpu::note_launches(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
extern "C" long long smip_kernel_launches(void) { return g_launches.load(); }

extern "C" int smip_version(int* major, int* minor, int* patch)
{
    if (major) *major = 0;
    if (minor) *minor = 3;
    if (patch) *patch = 2;
    return SMIP_OK;
}

// ---------------------------------------------------------- device context
namespace {

struct DeviceCtx {
    float2* tw32 = nullptr;  // exp(-2 pi i k / 2^kTwLog), k < 2^(kTwLog-1)
    double2* tw64 = nullptr;
    dfc* twdf = nullptr;     // the same table as float-float (hi, lo)
    int num_sms = 0;
    // smip_batch_launch: the bispectrum work of many stacks as one persistent
    // launch.  Two slots alternate; each holds page-locked host copies of the
    // stack records, the work list and its control words, their device
    // copies, and a CUDA graph captured once for the slot's buffers: the
    // three host-to-device copies, then the persistent kernel.  A call fills
    // the host side and launches the graph; the graph is captured again only
    // when a slot's buffers grow.
    struct MultiSlot {
        unsigned char* h_recs = nullptr;
        int2* h_items = nullptr;
        int* h_ctrl = nullptr;
        unsigned char* d_recs = nullptr;
        int2* d_items = nullptr;
        int* d_ctrl = nullptr;
        size_t rec_cap = 0, item_cap = 0;
        cudaGraphExec_t exec = nullptr; // the graph for grid CTAs
        int grid = 0;
        cudaEvent_t ev_used = nullptr; // the slot's last launch has read its host buffers
        bool used = false;
    };
    std::shared_ptr<std::mutex> gmu = std::make_shared<std::mutex>();
    std::shared_ptr<MultiSlot> mslot = std::shared_ptr<MultiSlot>(new MultiSlot[2], std::default_delete<MultiSlot[]>());
    int mnext = 0;
    cudaStream_t mst = nullptr;     // the batch stream
    cudaEvent_t ev_mdone = nullptr; // the last batch launch has finished
};

std::mutex g_ctx_mu;
std::map<int, DeviceCtx> g_ctx;

int device_ctx(int dev, DeviceCtx** out)
{
    std::lock_guard<std::mutex> lk(g_ctx_mu);
    auto it = g_ctx.find(dev);
    if (it == g_ctx.end()) {
        DeviceCtx c;
        CUDA_TRY(cudaSetDevice(dev));
        CUDA_TRY(cudaDeviceGetAttribute(&c.num_sms, cudaDevAttrMultiProcessorCount, dev));
        const int n = 1 << (kTwLog - 1);
        std::vector<float2> t32(n);
        std::vector<double2> t64(n);
        for (int k = 0; k < n; ++k) {
            const double a = 2.0 * M_PI * (double)k / (double)(1 << kTwLog);
            t64[k] = make_double2(std::cos(a), -std::sin(a));
            t32[k] = make_float2((float)t64[k].x, (float)t64[k].y);
        }
        std::vector<dfc> tdf(n);
        for (int k = 0; k < n; ++k) {
            const float hx = (float)t64[k].x, hy = (float)t64[k].y;
            tdf[k].h = make_float2(hx, hy);
            tdf[k].l = make_float2((float)(t64[k].x - (double)hx), (float)(t64[k].y - (double)hy));
        }
        CUDA_TRY(cudaMalloc(&c.tw32, sizeof(float2) * n));
        CUDA_TRY(cudaMalloc(&c.tw64, sizeof(double2) * n));
        CUDA_TRY(cudaMalloc(&c.twdf, sizeof(dfc) * n));
        CUDA_TRY(cudaMemcpy(c.tw32, t32.data(), sizeof(float2) * n, cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(c.tw64, t64.data(), sizeof(double2) * n, cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(c.twdf, tdf.data(), sizeof(dfc) * n, cudaMemcpyHostToDevice));
        it = g_ctx.emplace(dev, c).first;
    }
    *out = &it->second;
    return SMIP_OK;
}

int ilog2(long v)
{
    int l = 0;
    while ((1L << l) < v)
        ++l;
    return l;
}

bool pow2(long v) { return v > 0 && (v & (v - 1)) == 0; }

size_t dtype_size(int dt)
{
    switch (dt) {
    case SMIP_U8: return 1;
    case SMIP_U16: return 2;
    case SMIP_F32: return 4;
    case SMIP_F64: return 8;
    default: return 0;
    }
}

int make_geometry(long W, long H, long bdepth, Geometry* g)
{
    if (W < 3 || H < 3 || W > kMaxSide || H > kMaxSide)
        return fail(SMIP_E_UNSUPPORTED, "frame size must be in [3, 1024] per axis");
    const int De = (int)(bdepth / 2) * 2;
    if (bdepth < 0)
        return fail(SMIP_E_INVALID_ARGUMENT, "bdepth must be non-negative");
    if (!bispec_depth_supported(De))
        return fail(SMIP_E_UNSUPPORTED, "bispectrum depth (rounded down to even) must be in [2, 64]");
    if (De >= W || De >= H)
        return fail(SMIP_E_UNSUPPORTED, "bispectrum depth must be smaller than the frame size");
    g->W = (int)W;
    g->H = (int)H;
    g->logW = ilog2(W);
    g->logH = ilog2(H);
    // radix-2 kernels for powers of two in [16, 512]; mixed radix otherwise
    g->generic = !(pow2(W) && pow2(H) && W >= 16 && H >= 16 && W <= (1 << kMaxLog) && H <= (1 << kMaxLog));
    g->hw = (int)W / 2 + 1;
    g->Hs = (int)H + (int)(H & 1);
    g->bs1 = (int)(H / 2) * 2 + 1;
    g->De = De;
    g->E = (De / 2 + 1) * (De + 1);
    g->base_size = (long long)g->hw * g->bs1 * g->E;
    g->pW = make_gen_plan((int)W);
    g->pH = make_gen_plan((int)H);
    return SMIP_OK;
}

// Generic path: twiddle tables exp(-2 pi i k / L), k < L, in float-float,
// FP32 and FP64.
int make_gen_tw(int L, GenTw* t)
{
    std::vector<double2> t64(L);
    std::vector<float2> t32(L);
    std::vector<dfc> tdf(L);
    for (int k = 0; k < L; ++k) {
        const double a = 2.0 * M_PI * (double)k / (double)L;
        t64[k] = make_double2(std::cos(a), -std::sin(a));
        const float hx = (float)t64[k].x, hy = (float)t64[k].y;
        t32[k] = make_float2(hx, hy);
        tdf[k].h = t32[k];
        tdf[k].l = make_float2((float)(t64[k].x - (double)hx), (float)(t64[k].y - (double)hy));
    }
    // the passes' index map (GenPlan::map): j | e0 << 16 per pass and output
    const GenPlan p = make_gen_plan(L);
    std::vector<unsigned> map((size_t)p.nf * L);
    for (int f = 0, Ns = 1; f < p.nf; Ns *= p.fac[f], ++f) {
        const int R = p.fac[f], step = L / (Ns * R);
        for (int o = 0; o < L; ++o) {
            const int k = o % Ns, t = o / Ns, q = t % R;
            map[(size_t)f * L + o] = (unsigned)((t / R) * Ns + k) | ((unsigned)((k + q * Ns) * step) << 16);
        }
    }
    CUDA_TRY(cudaMalloc(&t->map, sizeof(unsigned) * map.size()));
    CUDA_TRY(cudaMemcpy(t->map, map.data(), sizeof(unsigned) * map.size(), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMalloc(&t->df, sizeof(dfc) * L));
    CUDA_TRY(cudaMalloc(&t->f32, sizeof(float2) * L));
    CUDA_TRY(cudaMalloc(&t->f64, sizeof(double2) * L));
    CUDA_TRY(cudaMemcpy(t->df, tdf.data(), sizeof(dfc) * L, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(t->f32, t32.data(), sizeof(float2) * L, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(t->f64, t64.data(), sizeof(double2) * L, cudaMemcpyHostToDevice));
    return SMIP_OK;
}

void free_gen_tw(GenTw* t)
{
    if (t->df) cudaFree(t->df);
    if (t->f32) cudaFree(t->f32);
    if (t->f64) cudaFree(t->f64);
    if (t->map) cudaFree(t->map);
    *t = GenTw();
}

// phasereco.cpp:17-36, the reference's own host arithmetic
void next_reco_index(double& r, double& phi, int& i, int& j)
{
    const double dr = 1.0;
    const double dphi = 1.0 / (2.0 * M_PI * r);
    int ii = i, jj = j;
    while ((i == ii) && (j == jj)) {
        if ((phi += dphi) > 2.0 * M_PI) {
            phi = 0;
            r += dr;
        }
        ii = static_cast<int>(r * std::cos(phi));
        jj = static_cast<int>(r * std::sin(phi));
    }
    i = ii;
    j = jj;
}

// phasereco.h:56-68.  ring (optional): per visit the radius r at which
// NextRecoIndex made it (r grows by 1 per turn of the spiral).
std::vector<int2> reco_visits(double R, std::vector<int>* ring = nullptr)
{
    std::vector<int2> v;
    double r = 0.0, phi = 0.0;
    int i = 0, j = 0;
    while (r <= R) {
        next_reco_index(r, phi, i, j);
        v.push_back(make_int2(i, j));
        if (ring)
            ring->push_back((int)r);
    }
    return v;
}

template <typename T> void dfree(T*& p)
{
    if (p)
        cudaFree(p);
    p = nullptr;
}

// Buffers of one phase reconstruction.
struct Reco {
    Geometry g {};
    double R = -1.0;
    int2* visits = nullptr;
    int mode = 0;                 // 0: the reference's spiral walk; 1: ring-parallel estimator
    int* fring = nullptr;         // ring mode: per point the ring that set its phase (-1: none)
    int* rq = nullptr;            // ring mode: visit indices grouped by ring
    std::vector<int> roff;        // ring k: rq[roff[k] .. roff[k+1])
    int4* pvis = nullptr;         // per point: first three visit indices, visit count
    unsigned* rbits = nullptr;    // per visit: recent pair slots (bitmask)
    int* rcount = nullptr;
    unsigned short* rlist = nullptr;
    int nvisits = 0;
    double2* phases = nullptr;
    float2* phf = nullptr;
    float4* sums = nullptr;
    float2* plan = nullptr;       // nvisits x (De+1)^2 pair phasors
    int* cnt = nullptr;
    double* cons = nullptr;
    unsigned char* flags = nullptr;
    RecoJob* job = nullptr;
    ~Reco()
    {
        dfree(visits);
        dfree(fring);
        dfree(rq);
        dfree(pvis);
        dfree(rbits);
        dfree(rcount);
        dfree(rlist);
        dfree(phases);
        dfree(phf);
        dfree(sums);
        dfree(plan);
        dfree(cnt);
        dfree(cons);
        dfree(flags);
        dfree(job);
    }
    // Buffers and visit tables for radius `radius` (allocated once per stack,
    // the tables again only when the radius changes).
    int prepare(double radius, cudaStream_t st)
    {
        const size_t np = (size_t)g.W * g.H;
        if (!phases) {
            CUDA_TRY(cudaMalloc(&phases, sizeof(double2) * np));
            CUDA_TRY(cudaMalloc(&phf, sizeof(float2) * np));
            CUDA_TRY(cudaMalloc(&sums, sizeof(float4) * np));
            CUDA_TRY(cudaMalloc(&cnt, sizeof(int) * np));
            CUDA_TRY(cudaMalloc(&cons, sizeof(double) * np));
            CUDA_TRY(cudaMalloc(&flags, np));
            CUDA_TRY(cudaMalloc(&job, sizeof(RecoJob)));
        }
        if (radius != R) {
            std::vector<int> vring;
            std::vector<int2> v = reco_visits(radius, &vring);
            CUDA_TRY(cudaStreamSynchronize(st));
            dfree(rq);
            {   // ring lists: each point once per ring, in visit order
                const int nr = vring.empty() ? 1 : vring.back() + 1;
                std::vector<std::vector<int>> per(nr + 1);
                std::vector<int> seen(np, -1);
                const int qmin0 = -(g.W >> 1), qmin1 = -(g.H >> 1), qmax0 = g.W - 1 + qmin0, qmax1 = g.H - 1 + qmin1;
                for (size_t q = 0; q < v.size(); ++q) {
                    const int2 w = v[q];
                    if (w.x < qmin0 || w.x > qmax0 || w.y < qmin1 || w.y > qmax1)
                        continue;
                    const size_t p = (size_t)(w.x < 0 ? w.x + g.W : w.x) + (size_t)(w.y < 0 ? w.y + g.H : w.y) * g.W;
                    const int k = std::max(1, vring[q]);
                    if (seen[p] == k)
                        continue;
                    seen[p] = k;
                    per[k].push_back((int)q);
                }
                std::vector<int> flat;
                roff.assign(per.size() + 1, 0);
                for (size_t k = 0; k < per.size(); ++k) {
                    roff[k] = (int)flat.size();
                    flat.insert(flat.end(), per[k].begin(), per[k].end());
                }
                roff[per.size()] = (int)flat.size();
                CUDA_TRY(cudaMalloc(&rq, sizeof(int) * std::max<size_t>(1, flat.size())));
                if (!flat.empty())
                    CUDA_TRY(cudaMemcpy(rq, flat.data(), sizeof(int) * flat.size(), cudaMemcpyHostToDevice));
            }
            dfree(visits);
            dfree(plan);
            dfree(pvis);
            dfree(rbits);
            dfree(rcount);
            dfree(rlist);
            CUDA_TRY(cudaMalloc(&visits, sizeof(int2) * v.size()));
            CUDA_TRY(cudaMemcpyAsync(visits, v.data(), sizeof(int2) * v.size(), cudaMemcpyHostToDevice, st));
            nvisits = (int)v.size();
            const size_t nv = (size_t)(g.De + 1) * (g.De + 1);
            CUDA_TRY(cudaMalloc(&plan, sizeof(float2) * nv * v.size()));
            // each point's visits (the walk's order; a point may be visited again)
            std::vector<int4> pv(np, make_int4(-1, -1, -1, 0));
            const int pmin0 = -(g.W >> 1), pmin1 = -(g.H >> 1), pmax0 = g.W - 1 + pmin0, pmax1 = g.H - 1 + pmin1;
            for (size_t q = 0; q < v.size(); ++q) {
                const int2 w = v[q];
                if (w.x < pmin0 || w.x > pmax0 || w.y < pmin1 || w.y > pmax1)
                    continue;
                int4& e = pv[(size_t)(w.x < 0 ? w.x + g.W : w.x) + (size_t)(w.y < 0 ? w.y + g.H : w.y) * g.W];
                if (e.w == 0) e.x = (int)q;
                else if (e.w == 1) e.y = (int)q;
                else if (e.w == 2) e.z = (int)q;
                ++e.w;
            }
            CUDA_TRY(cudaMalloc(&pvis, sizeof(int4) * np));
            CUDA_TRY(cudaMemcpyAsync(pvis, pv.data(), sizeof(int4) * np, cudaMemcpyHostToDevice, st));
            const size_t nwords = (nv + 31) / 32;
            CUDA_TRY(cudaMalloc(&rbits, sizeof(unsigned) * nwords * v.size()));
            CUDA_TRY(cudaMalloc(&rcount, sizeof(int) * v.size()));
            CUDA_TRY(cudaMalloc(&rlist, sizeof(unsigned short) * kRecentMax * v.size()));
            R = radius;
        }
        if (mode == 1 && !fring)
            CUDA_TRY(cudaMalloc(&fring, sizeof(int) * np));
        return SMIP_OK;
    }
    int run(const float2* Bnorm, double radius, int* err, cudaStream_t st)
    {
        const size_t np = (size_t)g.W * g.H;
        if (int rc = prepare(radius, st))
            return rc;
        CUDA_TRY(cudaMemsetAsync(phases, 0, sizeof(double2) * np, st));
        // the spiral walk's phase map marks a point without a phase by NaN (all bits set)
        CUDA_TRY(cudaMemsetAsync(phf, mode == 1 ? 0 : 0xff, sizeof(float2) * np, st));
        CUDA_TRY(cudaMemsetAsync(cons, 0, sizeof(double) * np, st));
        RecoJob j;
        j.B = Bnorm;
        j.visits = visits;
        j.nvisits = nvisits;
        j.W = g.W;
        j.H = g.H;
        j.De = g.De;
        j.phases = phases;
        j.phf = phf;
        j.sums = sums;
        j.plan = plan;
        j.cnt = cnt;
        j.cons = cons;
        j.flags = flags;
        j.err = err;
        j.pvis = pvis;
        j.rbits = rbits;
        j.rcount = rcount;
        j.rlist = rlist;
        CUDA_TRY(cudaMemcpyAsync(job, &j, sizeof(RecoJob), cudaMemcpyHostToDevice, st));
        if (mode == 1) {
            CUDA_TRY(launch_ring_reco(job, fring, rq, roff, g.W, g.H, st));
        } else {
            CUDA_TRY(launch_phase_reco(job, 1, g.W, g.H, g.De, st));
        }
        return SMIP_OK;
    }
    int download(double* ph, unsigned char* fl, double* cs, cudaStream_t st)
    {
        const size_t np = (size_t)g.W * g.H;
        if (ph)
            CUDA_TRY(cudaMemcpyAsync(ph, phases, sizeof(double2) * np, cudaMemcpyDeviceToHost, st));
        if (fl)
            CUDA_TRY(cudaMemcpyAsync(fl, flags, np, cudaMemcpyDeviceToHost, st));
        if (cs)
            CUDA_TRY(cudaMemcpyAsync(cs, cons, sizeof(double) * np, cudaMemcpyDeviceToHost, st));
        return SMIP_OK;
    }
};

int check_dev_err(int* err_dev, cudaStream_t st)
{
    int e = 0;
    CUDA_TRY(cudaMemcpyAsync(&e, err_dev, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (e == SMIP_DEV_ERR_TIMEOUT)
        return fail(SMIP_E_TIMEOUT, "a bounded device wait expired; results of the affected batch are incomplete");
    if (e == SMIP_DEV_ERR_OUT_OF_RANGE)
        return fail(SMIP_E_OUT_OF_RANGE, "Bispectrum: element address out of bounds (get_element would throw)");
    return SMIP_OK;
}

} // namespace

// ------------------------------------------------------------------- stack
struct smip_stack {
    int device = 0;
    DeviceCtx* ctx = nullptr;
    cudaStream_t st = nullptr;
    bool own_stream = false;
    Geometry g {};
    long bdepth_req = 0;
    int Bf = 0;                   // frames per batch
    int fpc = 16;                 // frames per column-pass chunk
    int dtype = -1;               // frame dtype fixed by the first push
    int kvariant = 0;             // bispectrum kernel staging (smip_stack_set_kernel_config)
    int kmin_part = 0;            // frames per split-tile part at least (0: the kernel's 8)
    int mode = 0;                 // 0 unset, 1 frames, 2 spectra
    long nframes = 0;             // frames accumulated (incl. pending)
    int pending = 0;              // frames staged for the next batch
    bool has_ref = false;
    // optional CUDA-event timing of the bispectrum kernel (on this stream)
    bool timing = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_pool;
    size_t ev_used = 0;
    double k2_ms = 0.0;
    long k2_launches = 0;
    double k2_frames = 0.0;
    std::vector<int> ev_frames;
    // device buffers
    float2 *B = nullptr, *C = nullptr, *Bn = nullptr;
    double* P = nullptr;
    double* Ppart = nullptr;
    void* sum = nullptr;          // u64 (integer frames) or double
    // Two frame batches: the host->device (or device->device) copy of the next
    // batch runs on the copy stream cst while the kernels read the current one.
    void* stg[2] = { nullptr, nullptr };
    int cur = 0;                  // buffer being filled
    size_t stg_bytes = 0;         // bytes per frame the two buffers hold (they only grow)
    cudaStream_t cst = nullptr;   // copy stream
    cudaEvent_t ev_copied[2] = { nullptr, nullptr }; // copies into stg[i] done (on cst)
    cudaEvent_t ev_free[2] = { nullptr, nullptr };   // kernels done reading stg[i] (on st)
    bool free_rec[2] = { false, false };
    // A batch whose frames the row pass reads straight from mapped
    // page-locked host memory (the first full batch of a push, which no
    // earlier work could overlap with a copy); the row pass writes them into
    // stg[cur] for the later kernels.  ev_zc: that row pass is done, so the
    // copy stream's next transfer does not share the host link with it.
    const void* zc_src = nullptr;
    cudaEvent_t ev_zc = nullptr;
    double* spec_staging = nullptr; // spectra input (mode 2)
    void* ref = nullptr;          // raw frame 0 (room for 8 bytes per pixel, any frame type)
    double* ref_sq = nullptr;
    dfc* Gt = nullptr;            // row-FFT output, float-float
    float2 *T = nullptr, *S = nullptr, *R = nullptr;
    float* corr = nullptr;
    float* rowmax = nullptr;      // per frame and row: the correlation's maximum
    float2* kscratch = nullptr;   // bispectrum kernel: partial sums of split tiles
    int* ktile_cnt = nullptr;     // bispectrum kernel: parts finished per split tile
    int* shifts = nullptr;        // all frames, int2
    long shifts_cap = 0;
    int* err = nullptr;
    Reco reco;
    double2* Z = nullptr;
    double* pfull = nullptr;
    double* maxbuf = nullptr;
    GenTw twW, twH;               // generic path: twiddles of the row and column lengths
    // phase recovery and the final image: a high-priority stream
    cudaStream_t rst = nullptr;
    cudaEvent_t ev_reco = nullptr;
    // smip_batch_launch: the stack's per-frame kernels of the batch are done
    cudaEvent_t ev_dep = nullptr;

    ~smip_stack()
    {
        cudaSetDevice(device);
        if (st)
            cudaStreamSynchronize(st);
        if (rst) {
            cudaStreamSynchronize(rst);
            cudaStreamDestroy(rst);
        }
        if (ev_reco) cudaEventDestroy(ev_reco);
        if (ev_dep) cudaEventDestroy(ev_dep);
        dfree(B); dfree(C); dfree(Bn); dfree(P); dfree(Ppart);
        if (sum) cudaFree(sum);
        if (cst)
            cudaStreamSynchronize(cst);
        for (int i = 0; i < 2; ++i) {
            if (stg[i]) cudaFree(stg[i]);
            if (ev_copied[i]) cudaEventDestroy(ev_copied[i]);
            if (ev_free[i]) cudaEventDestroy(ev_free[i]);
        }
        if (ev_zc) cudaEventDestroy(ev_zc);
        if (cst)
            cudaStreamDestroy(cst);
        dfree(spec_staging);
        if (ref) cudaFree(ref);
        dfree(ref_sq); dfree(Gt); dfree(T); dfree(S); dfree(R); dfree(corr); dfree(rowmax); dfree(shifts); dfree(err);
        dfree(kscratch); dfree(ktile_cnt);
        dfree(Z); dfree(pfull); dfree(maxbuf);
        free_gen_tw(&twW);
        free_gen_tw(&twH);
        for (auto& e : ev_pool) {
            cudaEventDestroy(e.first);
            cudaEventDestroy(e.second);
        }
        if (own_stream && st)
            cudaStreamDestroy(st);
    }

    size_t frame_elems() const { return (size_t)g.W * g.H; }
    size_t half_elems() const { return (size_t)g.hw * g.H; }

    int alloc()
    {
        const size_t bs = (size_t)g.base_size;
        CUDA_TRY(cudaMalloc(&B, sizeof(float2) * bs));
        CUDA_TRY(cudaMalloc(&C, sizeof(float2) * bs));
        CUDA_TRY(cudaMemsetAsync(B, 0, sizeof(float2) * bs, st));
        CUDA_TRY(cudaMemsetAsync(C, 0, sizeof(float2) * bs, st));
        CUDA_TRY(cudaMalloc(&P, sizeof(double) * half_elems()));
        CUDA_TRY(cudaMemsetAsync(P, 0, sizeof(double) * half_elems(), st));
        const int nchunks = (Bf + fpc - 1) / fpc;
        CUDA_TRY(cudaMalloc(&Ppart, sizeof(double) * half_elems() * nchunks));
        CUDA_TRY(cudaMalloc(&sum, 8 * frame_elems()));
        CUDA_TRY(cudaMemsetAsync(sum, 0, 8 * frame_elems(), st));
        CUDA_TRY(cudaMalloc(&Gt, sizeof(dfc) * half_elems() * Bf));
        CUDA_TRY(cudaMalloc(&T, sizeof(float2) * half_elems() * Bf));
        CUDA_TRY(cudaMalloc(&S, sizeof(float2) * (size_t)g.hw * g.Hs * Bf));
        if (g.Hs != g.H) // the pitch's spare column is never written: keep it defined
            CUDA_TRY(cudaMemsetAsync(S, 0, sizeof(float2) * (size_t)g.hw * g.Hs * Bf, st));
        if (g.generic) {
            int rc = make_gen_tw(g.W, &twW);
            if (!rc)
                rc = make_gen_tw(g.H, &twH);
            if (rc)
                return rc;
            g.pW.map = twW.map;
            g.pH.map = twH.map;
        }
        CUDA_TRY(cudaMalloc(&R, sizeof(float2) * half_elems()));
        CUDA_TRY(cudaMalloc(&corr, sizeof(float) * frame_elems() * Bf));
        CUDA_TRY(cudaMalloc(&rowmax, sizeof(float) * g.H * Bf));
        CUDA_TRY(cudaMalloc(&ref_sq, sizeof(double)));
        CUDA_TRY(cudaMalloc(&err, sizeof(int)));
        CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));
        // Everything a job needs is allocated here, with the stack, so that a
        // pooled stack serves further jobs without allocating: an allocation
        // (and a free, which synchronises the device) in the middle of
        // serving stalls the request loop until the GPU drains.
        CUDA_TRY(cudaMalloc(&ref, 8 * frame_elems()));
        CUDA_TRY(cudaMalloc(&kscratch, bispec_scratch_bytes(ctx->num_sms)));
        CUDA_TRY(cudaMalloc(&ktile_cnt, sizeof(int) * bispec_tile_counters(ctx->num_sms)));
        CUDA_TRY(cudaMemsetAsync(ktile_cnt, 0, sizeof(int) * bispec_tile_counters(ctx->num_sms), st));
        return ensure_shift_cap(kShiftCap0);
    }

    // shifts of the first kShiftCap0 frames fit without growing the buffer
    static constexpr long kShiftCap0 = 65536;

    int ensure_shift_cap(long n)
    {
        if (n <= shifts_cap)
            return SMIP_OK;
        long cap = std::max<long>(n, std::max<long>(1024, 2 * shifts_cap));
        int* nb = nullptr;
        CUDA_TRY(cudaMalloc(&nb, sizeof(int) * 2 * cap));
        if (shifts)
            CUDA_TRY(cudaMemcpyAsync(nb, shifts, sizeof(int) * 2 * shifts_cap, cudaMemcpyDeviceToDevice, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        dfree(shifts);
        shifts = nb;
        shifts_cap = cap;
        return SMIP_OK;
    }

    // the two frame buffers, the copy stream and its events: made for the first
    // frames, remade only for frames of a larger element type than the buffers
    // hold (a smaller type reuses them)
    int ensure_staging(size_t fbytes)
    {
        if (!cst)
            CUDA_TRY(cudaStreamCreateWithFlags(&cst, cudaStreamNonBlocking));
        if (stg[0] && stg_bytes < fbytes) { // larger frames: the buffers' last kernels must be done
            CUDA_TRY(cudaStreamSynchronize(st));
            free_staging();
        }
        for (int i = 0; i < 2; ++i) {
            if (!stg[i]) {
                CUDA_TRY(cudaMalloc(&stg[i], fbytes * Bf));
                stg_bytes = fbytes;
            }
            if (!ev_copied[i])
                CUDA_TRY(cudaEventCreateWithFlags(&ev_copied[i], cudaEventDisableTiming));
            if (!ev_free[i])
                CUDA_TRY(cudaEventCreateWithFlags(&ev_free[i], cudaEventDisableTiming));
        }
        return SMIP_OK;
    }

    void free_staging()
    {
        if (cst)
            cudaStreamSynchronize(cst);
        for (int i = 0; i < 2; ++i) {
            if (stg[i])
                cudaFree(stg[i]);
            stg[i] = nullptr;
            free_rec[i] = false;
        }
        cur = 0;
        stg_bytes = 0;
    }

    // Host-side preparation of the pending batch: every allocation and
    // synchronisation happens here, so that issue_batch can be captured.
    int prepare_batch()
    {
        if (pending == 0)
            return SMIP_OK;
        if (mode != 2) {
            int rc = ensure_shift_cap(nframes);
            if (rc)
                return rc;
        }
        return SMIP_OK;
    }

    // The pending batch's device work on stream q (kernels and device copies
    // only).  wait_copies: order it after the batch's frame copies on cst
    // (a graph launch orders them outside the graph instead).  timed: CUDA
    // events around the bispectrum kernel.
    int issue_batch(cudaStream_t q, bool wait_copies, bool timed, bool with_bispec = true)
    {
        const int n = pending;
        const long first_index = nframes - n;
        if (mode == 2) {
            CUDA_TRY(launch_import_spectra(spec_staging, n, g, S, q));
        } else {
            const size_t fe = frame_elems();
            const bool first = !has_ref;
            void* staging = stg[cur];
            const void* zc = zc_src;
            zc_src = nullptr;
            if (wait_copies && !zc) {
                CUDA_TRY(cudaEventRecord(ev_copied[cur], cst));
                CUDA_TRY(cudaStreamWaitEvent(q, ev_copied[cur], 0));
            }
            if (first) {
                CUDA_TRY(cudaMemcpyAsync(ref, zc ? zc : staging, dtype_size(dtype) * fe, cudaMemcpyDefault, q));
                CUDA_TRY(launch_sumsq(dtype, ref, (long long)fe, ref_sq, q));
            }
            if (g.generic) { // mixed-radix transforms (frame sizes other than powers of two in [16, 512])
                if (zc) {
                    CUDA_TRY(launch_gen_row_pass(dtype, zc, (long long)fe, n, g, Gt, twW.df, q, staging));
                    CUDA_TRY(cudaEventRecord(ev_zc, q));
                    CUDA_TRY(cudaStreamWaitEvent(cst, ev_zc, 0));
                } else {
                    CUDA_TRY(launch_gen_row_pass(dtype, staging, (long long)fe, n, g, Gt, twW.df, q));
                }
                if (first)
                    CUDA_TRY(launch_gen_col_pass(1, Gt, S, R, R, T, Ppart, 1, fpc, 0, g, twH.df, twH.f32, q));
                CUDA_TRY(launch_gen_col_pass(0, Gt, S, R, nullptr, T, Ppart, n, fpc, first ? 1 : 0, g, twH.df, twH.f32,
                                             q));
                CUDA_TRY(launch_power_reduce(P, Ppart, (n + fpc - 1) / fpc, g, q));
                CUDA_TRY(launch_gen_xcorr_rows(T, corr, rowmax, n, g, twW.f32, q));
            } else {
                if (zc) {
                    CUDA_TRY(launch_row_pass(dtype, zc, (long long)fe, n, g, Gt, ctx->twdf, q, staging));
                    CUDA_TRY(cudaEventRecord(ev_zc, q));
                    CUDA_TRY(cudaStreamWaitEvent(cst, ev_zc, 0));
                } else {
                    CUDA_TRY(launch_row_pass(dtype, staging, (long long)fe, n, g, Gt, ctx->twdf, q));
                }
                if (first)
                    CUDA_TRY(launch_col_pass(1, Gt, S, R, R, T, Ppart, 1, fpc, 0, g, ctx->twdf, ctx->tw32, q));
                CUDA_TRY(launch_col_pass(0, Gt, S, R, nullptr, T, Ppart, n, fpc, first ? 1 : 0, g, ctx->twdf,
                                         ctx->tw32, q));
                CUDA_TRY(launch_power_reduce(P, Ppart, (n + fpc - 1) / fpc, g, q));
                CUDA_TRY(launch_xcorr_rows(T, corr, rowmax, n, g, ctx->tw32, q));
            }
            CUDA_TRY(launch_xcorr_shift(dtype, corr, rowmax, staging, (long long)fe, ref, ref_sq, n, first ? 1 : 0,
                                        g, shifts + 2 * first_index, q));
            CUDA_TRY(launch_saa_add(dtype, sum, staging, (long long)fe, n, first ? 1 : 0, shifts + 2 * first_index, g, q));
        }
        if (!with_bispec)
            return SMIP_OK;
        const BispecLaunch L = bispec_launch(n);
        if (timed) {
            if (ev_used == ev_pool.size()) {
                cudaEvent_t a, b;
                CUDA_TRY(cudaEventCreate(&a));
                CUDA_TRY(cudaEventCreate(&b));
                ev_pool.emplace_back(a, b);
                ev_frames.push_back(0);
            }
            CUDA_TRY(cudaEventRecord(ev_pool[ev_used].first, q));
        }
        CUDA_TRY(launch_bispec_accumulate(L, g, q));
        if (timed) {
            CUDA_TRY(cudaEventRecord(ev_pool[ev_used].second, q));
            ev_frames[ev_used] = n;
            ++ev_used;
        }
        return SMIP_OK;
    }

    // The bispectrum launch of a batch of n frames (spectra in S).
    BispecLaunch bispec_launch(int n) const
    {
        BispecLaunch L;
        L.S = S;
        L.nframes = n;
        L.B = B;
        L.C = C;
        L.err = err;
        L.num_sms = ctx->num_sms;
        L.scratch = kscratch;
        L.tile_cnt = ktile_cnt;
        L.variant = kvariant;
        L.min_part = kmin_part;
        return L;
    }

    // Host bookkeeping once the batch's work is issued and ev_free[cur] is
    // recorded after its last read of the frame buffer.
    void commit_batch()
    {
        if (mode != 2) {
            free_rec[cur] = true; // the copy stream refills this buffer after ev_free[cur]
            cur ^= 1;
            has_ref = true;
        }
        pending = 0;
    }

    int run_batch()
    {
        if (pending == 0)
            return SMIP_OK;
        int rc = prepare_batch();
        if (rc || (rc = issue_batch(st, true, timing)))
            return rc;
        if (mode != 2)
            CUDA_TRY(cudaEventRecord(ev_free[cur], st)); // the last reader of this buffer
        commit_batch();
        return SMIP_OK;
    }

    // folds the recorded event pairs into the totals (stream must be idle)
    int collect_timing()
    {
        for (size_t q = 0; q < ev_used; ++q) {
            float ms = 0.f;
            CUDA_TRY(cudaEventElapsedTime(&ms, ev_pool[q].first, ev_pool[q].second));
            k2_ms += ms;
            k2_frames += ev_frames[q];
            ++k2_launches;
        }
        ev_used = 0;
        return SMIP_OK;
    }
};

static int check_stack(smip_stack_t s)
{
    if (!s)
        return fail(SMIP_E_INVALID_ARGUMENT, "null stack handle");
    if (cudaSetDevice(s->device) != cudaSuccess)
        return fail(SMIP_E_CUDA, "cudaSetDevice failed");
    return SMIP_OK;
}

extern "C" int smip_stack_create(smip_stack_t* out, int device, long ncols, long nrows, long bdepth, void* stream,
                                 long batch_frames)
{
    if (!out)
        return fail(SMIP_E_INVALID_ARGUMENT, "out is null");
    *out = nullptr;
    Geometry g;
    int rc = make_geometry(ncols, nrows, bdepth, &g);
    if (rc)
        return rc;
    DeviceCtx* ctx = nullptr;
    rc = device_ctx(device, &ctx);
    if (rc)
        return rc;
    smip_stack* s = new smip_stack();
    s->device = device;
    s->ctx = ctx;
    s->g = g;
    s->bdepth_req = bdepth;
    if (batch_frames <= 0) {
        // ~2 GB of per-batch buffers (float-float row spectra, spectra,
        // correlation columns and rows, frames), at most 1024 frames: larger
        // batches amortise the bispectrum's read-modify-write and split the
        // bispectrum kernel's work more evenly (measured by the autotuner:
        // 1024 beats 256 by 5 % at 256x256, 13 % at 128x128, 36 % at 64x64)
        const size_t per = (size_t)g.hw * g.H * (sizeof(dfc) + 2 * sizeof(float2)) + (size_t)g.W * g.H * (4 + 8);
        const long bf = (long)((2ull << 30) / per);
        batch_frames = std::min<long>(1024, std::max<long>(16, bf / 16 * 16));
    }
    s->Bf = (int)batch_frames;
    if (stream) {
        s->st = static_cast<cudaStream_t>(stream);
    } else {
        if (cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking) != cudaSuccess) {
            delete s;
            return fail(SMIP_E_CUDA, "cudaStreamCreate failed");
        }
        s->own_stream = true;
    }
    rc = s->alloc();
    if (rc) {
        delete s;
        return rc;
    }
    *out = s;
    return SMIP_OK;
}

extern "C" int smip_stack_destroy(smip_stack_t s)
{
    if (!s)
        return SMIP_OK;
    delete s;
    return SMIP_OK;
}

extern "C" int smip_stack_push_frames(smip_stack_t s, const void* frames, int dtype, long count, long stride_bytes,
                                      int on_device)
{
    int rc = check_stack(s);
    if (rc)
        return rc;
    const size_t es = dtype_size(dtype);
    if (!es)
        return fail(SMIP_E_INVALID_ARGUMENT, "unknown frame dtype");
    if (count < 0 || (count > 0 && !frames))
        return fail(SMIP_E_INVALID_ARGUMENT, "invalid frame buffer");
    if (s->mode == 2)
        return fail(SMIP_E_INVALID_ARGUMENT, "stack accumulates spectra; frames cannot be mixed in");
    if (s->dtype >= 0 && s->dtype != dtype) {
        if (s->nframes != 0)
            return fail(SMIP_E_INVALID_ARGUMENT, "frame dtype differs from the stack's first frames");
        s->dtype = -1; // after a reset: a new element type (ensure_staging keeps big enough buffers)
    }
    const size_t fbytes = es * s->frame_elems();
    if (stride_bytes == 0)
        stride_bytes = (long)fbytes;
    if ((size_t)stride_bytes < fbytes)
        return fail(SMIP_E_INVALID_ARGUMENT, "frame stride smaller than a frame");
    if (s->dtype < 0) {
        if ((rc = s->ensure_staging(fbytes)))
            return rc;
        s->dtype = dtype;
    }
    s->mode = 1;
    const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    const char* src = static_cast<const char*>(frames);
    // page-locked host frames: the first full batch is read by the row pass
    // through the mapped pointer instead of waiting for a copy
    const char* mapped = nullptr;
    if (!on_device && (size_t)stride_bytes == fbytes && s->pending == 0 && count >= s->Bf) {
        cudaPointerAttributes pa {};
        if (cudaPointerGetAttributes(&pa, frames) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer)
            mapped = static_cast<const char*>(pa.devicePointer);
        else
            cudaGetLastError(); // pageable memory: not an error
        if (mapped && !s->ev_zc)
            CUDA_TRY(cudaEventCreateWithFlags(&s->ev_zc, cudaEventDisableTiming));
    }
    long done = 0;
    if (mapped) {
        s->zc_src = mapped;
        s->pending = s->Bf;
        s->nframes += s->Bf;
        done = s->Bf;
        if ((rc = s->run_batch())) {
            s->zc_src = nullptr;
            return rc;
        }
    }
    while (done < count) {
        const long k = std::min<long>(count - done, s->Bf - s->pending);
        if (s->pending == 0 && s->free_rec[s->cur]) // the kernels of the buffer's last batch are done with it
            CUDA_TRY(cudaStreamWaitEvent(s->cst, s->ev_free[s->cur], 0));
        char* dst = static_cast<char*>(s->stg[s->cur]) + fbytes * s->pending;
        if ((size_t)stride_bytes == fbytes)
            CUDA_TRY(cudaMemcpyAsync(dst, src + done * stride_bytes, fbytes * k, kind, s->cst));
        else
            CUDA_TRY(cudaMemcpy2DAsync(dst, fbytes, src + done * stride_bytes, stride_bytes, fbytes, k, kind, s->cst));
        s->pending += (int)k;
        s->nframes += k;
        done += k;
        if (s->pending == s->Bf) {
            rc = s->run_batch();
            if (rc)
                return rc;
        }
    }
    return SMIP_OK;
}

extern "C" int smip_stack_set_kernel_config(smip_stack_t s, int variant, int min_part_frames)
{
    int rc = check_stack(s);
    if (rc)
        return rc;
    if (variant < 0 || variant > 1 || min_part_frames < 0)
        return fail(SMIP_E_INVALID_ARGUMENT, "kernel variant must be 0 or 1 and min_part_frames >= 0");
    s->kvariant = variant;
    s->kmin_part = min_part_frames;
    return SMIP_OK;
}

extern "C" int smip_stack_set_reco_mode(smip_stack_t s, int mode)
{
    int rc = check_stack(s);
    if (rc)
        return rc;
    if (mode != SMIP_RECO_SPIRAL && mode != SMIP_RECO_RINGS)
        return fail(SMIP_E_INVALID_ARGUMENT, "unknown phase-recovery mode");
    s->reco.mode = mode; // read on the host when the next reconstruction is issued
    return SMIP_OK;
}

extern "C" int smip_stack_accumulate_fft(smip_stack_t s, const double* spectra, long count, int on_device)
{
    int rc = check_stack(s);
    if (rc)
        return rc;
    if (count < 0 || (count > 0 && !spectra))
        return fail(SMIP_E_INVALID_ARGUMENT, "invalid spectrum buffer");
    if (s->mode == 1)
        return fail(SMIP_E_INVALID_ARGUMENT, "stack accumulates frames; spectra cannot be mixed in");
    const size_t sbytes = sizeof(double) * 2 * s->frame_elems();
    if (!s->spec_staging)
        CUDA_TRY(cudaMalloc(&s->spec_staging, sbytes * s->Bf));
    s->mode = 2;
    const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    long done = 0;
    while (done < count) {
        const long k = std::min<long>(count - done, s->Bf - s->pending);
        CUDA_TRY(cudaMemcpyAsync(reinterpret_cast<char*>(s->spec_staging) + sbytes * s->pending,
                                 reinterpret_cast<const char*>(spectra) + sbytes * done, sbytes * k, kind, s->st));
        s->pending += (int)k;
        s->nframes += k;
        done += k;
        if (s->pending == s->Bf) {
            rc = s->run_batch();
            if (rc)
                return rc;
        }
    }
    return SMIP_OK;
}

extern "C" int smip_stack_reset(smip_stack_t s)
{
    int rc = check_stack(s);
    if (rc)
        return rc;
    CUDA_TRY(cudaStreamSynchronize(s->st));
    if (s->cst) // frames copied for a batch that the reset drops
        CUDA_TRY(cudaStreamSynchronize(s->cst));
    if ((rc = s->collect_timing()))
        return rc;
    const size_t bs = (size_t)s->g.base_size;
    CUDA_TRY(cudaMemsetAsync(s->B, 0, sizeof(float2) * bs, s->st));
    CUDA_TRY(cudaMemsetAsync(s->C, 0, sizeof(float2) * bs, s->st));
    CUDA_TRY(cudaMemsetAsync(s->P, 0, sizeof(double) * s->half_elems(), s->st));
    CUDA_TRY(cudaMemsetAsync(s->sum, 0, 8 * s->frame_elems(), s->st));
    CUDA_TRY(cudaMemsetAsync(s->err, 0, sizeof(int), s->st));
    if (s->ktile_cnt) // a launch that stopped early (timeout) may leave parts counted
        CUDA_TRY(cudaMemsetAsync(s->ktile_cnt, 0, sizeof(int) * bispec_tile_counters(s->ctx->num_sms), s->st));
    s->nframes = 0;
    s->pending = 0;
    s->has_ref = false;
    s->mode = 0;
    return SMIP_OK;
}

extern "C" int smip_stack_set_timing(smip_stack_t s, int on)
{
    int rc = check_stack(s);
    if (rc)
        return rc;
    s->timing = on != 0;
    return SMIP_OK;
}

extern "C" int smip_stack_kernel_time(smip_stack_t s, double* bispec_ms, long* launches, double* frames)
{
    int rc = check_stack(s);
    if (rc)
        return rc;
    CUDA_TRY(cudaStreamSynchronize(s->st));
    if ((rc = s->collect_timing()))
        return rc;
    if (bispec_ms) *bispec_ms = s->k2_ms;
    if (launches) *launches = s->k2_launches;
    if (frames) *frames = s->k2_frames;
    s->k2_ms = 0.0;
    s->k2_launches = 0;
    s->k2_frames = 0.0;
    return SMIP_OK;
}

extern "C" int smip_stack_flush(smip_stack_t s)
{
    int rc = check_stack(s);
    if (rc)
        return rc;
    return s->run_batch();
}

extern "C" int smip_stack_sync(smip_stack_t s)
{
    int rc = smip_stack_flush(s);
    if (rc)
        return rc;
    return check_dev_err(s->err, s->st);
}

// The pending batches of several stacks: each stack's per-frame kernels on
// its own stream (concurrently), then the bispectrum work of all of them as
// one persistent launch over a work list of every stack's units, longest
// first (launch_bispec_multi), run by a CUDA graph captured once per slot
// buffer set (the records and the work list travel in device memory).  Each
// unit is what the stack's own launch would run, so results are identical to
// smip_stack_flush on each stack.
static int multi_slot_reserve(DeviceCtx::MultiSlot& m, size_t nrec, size_t nitem)
{
    if (nrec <= m.rec_cap && nitem <= m.item_cap)
        return SMIP_OK;
    if (m.used)
        CUDA_TRY(cudaEventSynchronize(m.ev_used));
    if (m.exec) {
        cudaGraphExecDestroy(m.exec);
        m.exec = nullptr;
    }
    const size_t rb = bispec_multi_rec_bytes();
    if (nrec > m.rec_cap) {
        if (m.h_recs) cudaFreeHost(m.h_recs);
        if (m.d_recs) cudaFree(m.d_recs);
        m.h_recs = m.d_recs = nullptr;
        m.rec_cap = std::max<size_t>(nrec, 2 * m.rec_cap);
        CUDA_TRY(cudaMallocHost(&m.h_recs, rb * m.rec_cap));
        CUDA_TRY(cudaMalloc(&m.d_recs, rb * m.rec_cap));
    }
    if (nitem > m.item_cap) {
        if (m.h_items) cudaFreeHost(m.h_items);
        if (m.d_items) cudaFree(m.d_items);
        m.h_items = m.d_items = nullptr;
        m.item_cap = std::max<size_t>(nitem, 2 * m.item_cap);
        CUDA_TRY(cudaMallocHost(&m.h_items, sizeof(int2) * m.item_cap));
        CUDA_TRY(cudaMalloc(&m.d_items, sizeof(int2) * m.item_cap));
    }
    if (!m.h_ctrl) {
        CUDA_TRY(cudaMallocHost(&m.h_ctrl, 2 * sizeof(int)));
        CUDA_TRY(cudaMalloc(&m.d_ctrl, 2 * sizeof(int)));
    }
    return SMIP_OK;
}

extern "C" int smip_batch_launch(smip_stack_t* stacks, long count)
{
    return smip_batch_launch_reserve(stacks, count, 0);
}

extern "C" int smip_batch_launch_reserve(smip_stack_t* stacks, long count, int reserve_sms)
{
    if (count < 0 || (count > 0 && !stacks))
        return fail(SMIP_E_INVALID_ARGUMENT, "invalid stack list");
    std::vector<smip_stack*> L;
    for (long i = 0; i < count; ++i) {
        int rc = check_stack(stacks[i]);
        if (rc)
            return rc;
        if (stacks[i]->device != stacks[0]->device)
            return fail(SMIP_E_INVALID_ARGUMENT, "stacks must live on the same device");
        if (std::find(L.begin(), L.end(), stacks[i]) != L.end())
            return fail(SMIP_E_INVALID_ARGUMENT, "a stack appears twice in the list");
        if (stacks[i]->pending > 0)
            L.push_back(stacks[i]);
    }
    if (L.empty())
        return SMIP_OK;
    DeviceCtx* ctx = L[0]->ctx;
    if (reserve_sms < 0 || reserve_sms >= ctx->num_sms)
        return fail(SMIP_E_INVALID_ARGUMENT, "reserve_sms must be in [0, SM count)");
    const int grid = ctx->num_sms - reserve_sms;
    std::lock_guard<std::mutex> lk(*ctx->gmu);
    CUDA_TRY(cudaSetDevice(L[0]->device));
    if (!ctx->mst) {
        CUDA_TRY(cudaStreamCreateWithFlags(&ctx->mst, cudaStreamNonBlocking));
        CUDA_TRY(cudaEventCreateWithFlags(&ctx->ev_mdone, cudaEventDisableTiming));
        for (int k = 0; k < 2; ++k)
            CUDA_TRY(cudaEventCreateWithFlags(&ctx->mslot.get()[k].ev_used, cudaEventDisableTiming));
    }
    // 1. every stack's per-frame kernels on its own stream
    std::vector<int> npend(L.size());
    for (size_t k = 0; k < L.size(); ++k) {
        smip_stack* s = L[k];
        npend[k] = s->pending;
        int rc = s->prepare_batch();
        if (!rc)
            rc = s->issue_batch(s->st, true, false, false);
        if (rc)
            return rc;
        if (s->mode != 2)
            CUDA_TRY(cudaEventRecord(s->ev_free[s->cur], s->st)); // the frames' last reader
        if (!s->ev_dep)
            CUDA_TRY(cudaEventCreateWithFlags(&s->ev_dep, cudaEventDisableTiming));
        CUDA_TRY(cudaEventRecord(s->ev_dep, s->st));
    }
    // 2. records and the work list, in the next slot's host buffers
    DeviceCtx::MultiSlot& m = ctx->mslot.get()[ctx->mnext];
    ctx->mnext ^= 1;
    if (m.used)
        CUDA_TRY(cudaEventSynchronize(m.ev_used)); // its previous launch has copied the host buffers
    const size_t rb = bispec_multi_rec_bytes();
    std::vector<std::vector<int>> uf(L.size());
    std::vector<unsigned char> recs(rb * L.size());
    size_t nitems = 0;
    for (size_t k = 0; k < L.size(); ++k) {
        const int units = bispec_multi_fill(recs.data() + rb * k, L[k]->bispec_launch(npend[k]), L[k]->g, &uf[k]);
        if (units < 0)
            return fail(SMIP_E_CUDA, "tensor map encoding failed");
        nitems += (size_t)units;
    }
    int rc = multi_slot_reserve(m, L.size(), nitems);
    if (rc)
        return rc;
    std::memcpy(m.h_recs, recs.data(), recs.size());
    {   // longest units first (frames per unit), ties in stack and unit order
        std::vector<std::pair<int, int2>> it;
        it.reserve(nitems);
        for (size_t k = 0; k < L.size(); ++k)
            for (size_t u = 0; u < uf[k].size(); ++u)
                it.push_back({ uf[k][u], make_int2((int)k, (int)u) });
        std::stable_sort(it.begin(), it.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
        for (size_t q = 0; q < nitems; ++q)
            m.h_items[q] = it[q].second;
    }
    m.h_ctrl[0] = (int)nitems;
    m.h_ctrl[1] = 0;
    // 3. the slot's graph on the batch stream, after every stack's per-frame kernels
    for (smip_stack* s : L)
        CUDA_TRY(cudaStreamWaitEvent(ctx->mst, s->ev_dep, 0));
    if (m.exec && m.grid != grid) { // another grid size: capture again
        CUDA_TRY(cudaEventSynchronize(m.ev_used));
        cudaGraphExecDestroy(m.exec);
        m.exec = nullptr;
    }
    if (!m.exec) {
        cudaGraph_t graph = nullptr;
        CUDA_TRY(cudaStreamBeginCapture(ctx->mst, cudaStreamCaptureModeRelaxed));
        cudaError_t ce = cudaMemcpyAsync(m.d_recs, m.h_recs, rb * m.rec_cap, cudaMemcpyHostToDevice, ctx->mst);
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(m.d_items, m.h_items, sizeof(int2) * m.item_cap, cudaMemcpyHostToDevice, ctx->mst);
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(m.d_ctrl, m.h_ctrl, 2 * sizeof(int), cudaMemcpyHostToDevice, ctx->mst);
        if (ce == cudaSuccess)
            ce = launch_bispec_multi(m.d_recs, m.d_items, m.d_ctrl, grid, ctx->mst);
        const cudaError_t ee = cudaStreamEndCapture(ctx->mst, &graph);
        if (ce == cudaSuccess && ee == cudaSuccess)
            ce = cudaGraphInstantiate(&m.exec, graph, 0);
        if (graph)
            cudaGraphDestroy(graph);
        if (ce != cudaSuccess || ee != cudaSuccess) {
            cudaGetLastError();
            m.exec = nullptr;
            return fail(SMIP_E_CUDA, cudaGetErrorString(ce != cudaSuccess ? ce : ee));
        }
        m.grid = grid;
    }
    CUDA_TRY(cudaGraphLaunch(m.exec, ctx->mst));
    CUDA_TRY(cudaEventRecord(m.ev_used, ctx->mst));
    m.used = true;
    CUDA_TRY(cudaEventRecord(ctx->ev_mdone, ctx->mst));
    for (smip_stack* s : L) {
        // the stack's later work (its next batch overwrites the spectra) follows the launch
        CUDA_TRY(cudaStreamWaitEvent(s->st, ctx->ev_mdone, 0));
        s->commit_batch();
    }
    return SMIP_OK;
}

extern "C" int smip_diag_bounded_wait(int device, double timeout_s)
{
    if (!(timeout_s > 0.0 && timeout_s <= 10.0))
        return fail(SMIP_E_INVALID_ARGUMENT, "timeout must be in (0, 10] s");
    CUDA_TRY(cudaSetDevice(device));
    cudaStream_t st = nullptr;
    int* buf = nullptr; // [0] device error word, [1] the flag nothing sets
    CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    int rc = SMIP_OK;
    cudaError_t e = cudaMalloc(&buf, 2 * sizeof(int));
    if (e == cudaSuccess)
        e = cudaMemsetAsync(buf, 0, 2 * sizeof(int), st);
    if (e == cudaSuccess)
        e = launch_bounded_wait_probe(buf, buf + 1, timeout_s, st);
    if (e != cudaSuccess)
        rc = fail(SMIP_E_CUDA, cudaGetErrorString(e));
    else
        rc = check_dev_err(buf, st); // SMIP_E_TIMEOUT, as after any expired wait
    cudaStreamSynchronize(st);
    if (buf)
        cudaFree(buf);
    cudaStreamDestroy(st);
    return rc;
}

extern "C" int smip_stack_frame_count(smip_stack_t s, long* n)
{
    int rc = check_stack(s);
    if (rc)
        return rc;
    if (n)
        *n = s->nframes;
    return SMIP_OK;
}

extern "C" int smip_stack_bispectrum_size(smip_stack_t s, long* n)
{
    int rc = check_stack(s);
    if (rc)
        return rc;
    if (n)
        *n = (long)s->g.base_size;
    return SMIP_OK;
}

extern "C" int smip_stack_shifts(smip_stack_t s, int* xy, long first, long count)
{
    int rc = smip_stack_sync(s);
    if (rc)
        return rc;
    if (s->mode != 1)
        return fail(SMIP_E_BAD_CALL, "no frames have been correlated");
    if (first < 0 || count < 0 || first + count > s->nframes)
        return fail(SMIP_E_OUT_OF_RANGE, "frame range outside the stack");
    CUDA_TRY(cudaMemcpyAsync(xy, s->shifts + 2 * first, sizeof(int) * 2 * count, cudaMemcpyDeviceToHost, s->st));
    CUDA_TRY(cudaStreamSynchronize(s->st));
    return SMIP_OK;
}

static int need_frames(smip_stack_t s)
{
    if (s->nframes == 0)
        return fail(SMIP_E_RUNTIME, "division by zero: no frames accumulated");
    return SMIP_OK;
}

extern "C" int smip_stack_sum(smip_stack_t s, double* out)
{
    int rc = smip_stack_sync(s);
    if (rc || (rc = need_frames(s)))
        return rc;
    if (s->mode != 1)
        return fail(SMIP_E_BAD_CALL, "no frames have been added to the sum");
    const size_t n = s->frame_elems();
    std::vector<uint64_t> raw(n);
    CUDA_TRY(cudaMemcpyAsync(raw.data(), s->sum, 8 * n, cudaMemcpyDeviceToHost, s->st));
    CUDA_TRY(cudaStreamSynchronize(s->st));
    const double nf = (double)s->nframes;
    if (s->dtype == SMIP_U8 || s->dtype == SMIP_U16) {
        for (size_t i = 0; i < n; ++i)
            out[i] = (double)raw[i] / nf; // exact integer sum, as the reference's double sum
    } else {
        for (size_t i = 0; i < n; ++i) {
            double v;
            std::memcpy(&v, &raw[i], 8);
            out[i] = v / nf;
        }
    }
    return SMIP_OK;
}

extern "C" int smip_stack_power(smip_stack_t s, double* out)
{
    int rc = smip_stack_sync(s);
    if (rc || (rc = need_frames(s)))
        return rc;
    if (!s->pfull)
        CUDA_TRY(cudaMalloc(&s->pfull, sizeof(double) * s->frame_elems()));
    const double pnorm = (double)((size_t)s->nframes * s->frame_elems());
    CUDA_TRY(launch_power_full(s->P, pnorm, s->g, s->pfull, s->st));
    CUDA_TRY(cudaMemcpyAsync(out, s->pfull, sizeof(double) * s->frame_elems(), cudaMemcpyDeviceToHost, s->st));
    CUDA_TRY(cudaStreamSynchronize(s->st));
    return SMIP_OK;
}

// The reconstruction's stream (high priority) and its buffers: the
// normalised bispectrum, the final image and the phase recovery's buffers
// and visit tables for radius R.
static int prepare_reco(smip_stack_t s, double R)
{
    if (!s->rst) {
        int least = 0, greatest = 0;
        CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        CUDA_TRY(cudaStreamCreateWithPriority(&s->rst, cudaStreamNonBlocking, greatest));
        CUDA_TRY(cudaEventCreateWithFlags(&s->ev_reco, cudaEventDisableTiming));
    }
    if (!s->Bn)
        CUDA_TRY(cudaMalloc(&s->Bn, sizeof(float2) * s->g.base_size));
    if (!s->Z) {
        CUDA_TRY(cudaMalloc(&s->Z, sizeof(double2) * s->frame_elems()));
        CUDA_TRY(cudaMalloc(&s->maxbuf, sizeof(double)));
    }
    s->reco.g = s->g;
    return s->reco.prepare(R, s->rst);
}

static int normalize_bispec(smip_stack_t s, cudaStream_t q)
{
    if (!s->Bn)
        CUDA_TRY(cudaMalloc(&s->Bn, sizeof(float2) * s->g.base_size));
    CUDA_TRY(launch_bispec_normalize(s->B, s->C, (double)s->nframes, s->g.base_size, s->Bn, q));
    return SMIP_OK;
}

extern "C" int smip_stack_bispectrum(smip_stack_t s, float* out)
{
    int rc = smip_stack_sync(s);
    if (rc || (rc = need_frames(s)))
        return rc;
    if ((rc = normalize_bispec(s, s->st)))
        return rc;
    CUDA_TRY(cudaMemcpyAsync(out, s->Bn, sizeof(float2) * s->g.base_size, cudaMemcpyDeviceToHost, s->st));
    CUDA_TRY(cudaStreamSynchronize(s->st));
    return SMIP_OK;
}

// Phase recovery (and the final image) run on the stack's high-priority
// stream: the walk is one CTA per job, and when several jobs share the GPU
// its blocks are scheduled ahead of pending accumulation blocks of other
// jobs.  The stack's stream is idle here (synchronised); rejoin_stream
// orders the later downloads on it after this work.
static int stack_reco(smip_stack_t s, double R)
{
    int rc = smip_stack_sync(s);
    if (rc || (rc = need_frames(s)))
        return rc;
    if (!(R >= 0.0))
        return fail(SMIP_E_INVALID_ARGUMENT, "reco_radius must be >= 0");
    if ((rc = prepare_reco(s, R)) || (rc = normalize_bispec(s, s->rst)))
        return rc;
    return s->reco.run(s->Bn, R, s->err, s->rst);
}

static int rejoin_stream(smip_stack_t s)
{
    CUDA_TRY(cudaEventRecord(s->ev_reco, s->rst));
    CUDA_TRY(cudaStreamWaitEvent(s->st, s->ev_reco, 0));
    return SMIP_OK;
}

extern "C" int smip_stack_reconstruct(smip_stack_t s, double R, double* phases, unsigned char* flags, double* cons)
{
    int rc = stack_reco(s, R);
    if (rc || (rc = rejoin_stream(s)))
        return rc;
    if ((rc = s->reco.download(phases, flags, cons, s->st)))
        return rc;
    return check_dev_err(s->err, s->st);
}

extern "C" int smip_stack_finish(smip_stack_t s, double R, double* image, double* phases, unsigned char* flags,
                                 double* cons)
{
    int rc = stack_reco(s, R);
    if (rc)
        return rc;
    if (s->mode != 1)
        return fail(SMIP_E_BAD_CALL, "the final image needs the power spectrum of pushed frames");
    if (!(R > 0.0))
        return fail(SMIP_E_DOMAIN, "WindowFunction aperture size <= 0");
    const size_t n = s->frame_elems();
    const double pnorm = (double)((size_t)s->nframes * n);
    CUDA_TRY(launch_finish(s->P, pnorm, s->reco.phases, 2.0 * R, s->g, s->Z, nullptr, s->maxbuf, s->ctx->tw64, s->rst,
                           s->twW.f64, s->twH.f64));
    if ((rc = rejoin_stream(s)))
        return rc;
    if (image)
        CUDA_TRY(cudaMemcpyAsync(image, s->Z, sizeof(double2) * n, cudaMemcpyDeviceToHost, s->st));
    if ((rc = s->reco.download(phases, flags, cons, s->st)))
        return rc;
    return check_dev_err(s->err, s->st);
}

extern "C" int smip_stack_prepare_reco(smip_stack_t s, double reco_radius)
{
    int rc = check_stack(s);
    if (rc)
        return rc;
    if (!(reco_radius >= 0.0))
        return fail(SMIP_E_INVALID_ARGUMENT, "reco_radius must be >= 0");
    CUDA_TRY(cudaSetDevice(s->device));
    if ((rc = prepare_reco(s, reco_radius)))
        return rc;
    CUDA_TRY(cudaStreamSynchronize(s->rst)); // the visit tables' copies
    return SMIP_OK;
}

extern "C" int smip_stack_share_reference(smip_stack_t dst, smip_stack_t src)
{
    int rc = smip_stack_sync(dst);
    if (rc)
        return rc;
    if (!src || src->device != dst->device)
        return fail(SMIP_E_INVALID_ARGUMENT, "stacks must live on the same device");
    if (!dst->has_ref)
        return fail(SMIP_E_BAD_CALL, "dst has no reference frame yet");
    if (src->g.W != dst->g.W || src->g.H != dst->g.H || src->g.De != dst->g.De)
        return fail(SMIP_E_INVALID_ARGUMENT, "Bispectrum::operator+=(const Bispectrum) : operand dimension size mismatch");
    if (src->nframes != 0)
        return fail(SMIP_E_BAD_CALL, "src already holds frames");
    const size_t fbytes = dtype_size(dst->dtype) * dst->frame_elems();
    src->dtype = dst->dtype;
    src->mode = 1;
    if (int rc2 = src->ensure_staging(fbytes))
        return rc2;
    CUDA_TRY(cudaMemcpy(src->ref, dst->ref, fbytes, cudaMemcpyDeviceToDevice));
    CUDA_TRY(cudaMemcpy(src->R, dst->R, sizeof(float2) * dst->half_elems(), cudaMemcpyDeviceToDevice));
    CUDA_TRY(cudaMemcpy(src->ref_sq, dst->ref_sq, sizeof(double), cudaMemcpyDeviceToDevice));
    src->has_ref = true;
    return SMIP_OK;
}

__global__ void add_u64_kernel(unsigned long long* d, const unsigned long long* s, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        d[i] += s[i];
}
__global__ void add_f64_kernel(double* d, const double* s, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        d[i] += s[i];
}

extern "C" int smip_stack_merge(smip_stack_t dst, smip_stack_t src)
{
    int rc = smip_stack_sync(dst);
    if (rc || (rc = smip_stack_sync(src)))
        return rc;
    if (src->device != dst->device)
        return fail(SMIP_E_INVALID_ARGUMENT, "stacks must live on the same device");
    if (src->g.W != dst->g.W || src->g.H != dst->g.H || src->g.De != dst->g.De)
        return fail(SMIP_E_INVALID_ARGUMENT, "Bispectrum::operator+=(const Bispectrum) : operand dimension size mismatch");
    if (src->mode != dst->mode || (src->mode == 1 && src->dtype != dst->dtype))
        return fail(SMIP_E_INVALID_ARGUMENT, "stacks accumulate different inputs");
    CUDA_TRY(launch_bispec_merge(dst->B, dst->C, src->B, src->C, dst->g.base_size, dst->st));
    add_f64_kernel<<<256, 256, 0, dst->st>>>(dst->P, src->P, (long long)dst->half_elems()); note_launches(1);
    if (dst->mode == 1) {
        if (dst->dtype == SMIP_U8 || dst->dtype == SMIP_U16)
            add_u64_kernel<<<256, 256, 0, dst->st>>>((unsigned long long*)dst->sum, (const unsigned long long*)src->sum,
                                                     (long long)dst->frame_elems());
        else
            add_f64_kernel<<<256, 256, 0, dst->st>>>((double*)dst->sum, (const double*)src->sum,
                                                     (long long)dst->frame_elems());
        note_launches(1);
        rc = dst->ensure_shift_cap(dst->nframes + src->nframes);
        if (rc)
            return rc;
        CUDA_TRY(cudaMemcpyAsync(dst->shifts + 2 * dst->nframes, src->shifts, sizeof(int) * 2 * src->nframes,
                                 cudaMemcpyDeviceToDevice, dst->st));
    }
    dst->nframes += src->nframes;
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(dst->st));
    return SMIP_OK;
}

extern "C" int smip_stack_save_bispectrum(smip_stack_t s, const char* path)
{
    if (!path)
        return fail(SMIP_E_INVALID_ARGUMENT, "null path");
    long n = 0;
    int rc = smip_stack_bispectrum_size(s, &n);
    if (rc)
        return rc;
    std::vector<float> buf(2 * (size_t)n);
    if ((rc = smip_stack_bispectrum(s, buf.data())))
        return rc;
    FILE* f = std::fopen(path, "wb");
    if (!f)
        return fail(SMIP_E_RUNTIME, std::string("unable to open file ") + path + " for writing");
    // bispectrum.h:421-428: size_t base_size, 4 x size_t dims, T[base_size]
    const size_t hdr[5] = { (size_t)n, (size_t)s->g.W, (size_t)s->g.H, (size_t)s->bdepth_req, (size_t)s->bdepth_req };
    bool ok = std::fwrite(hdr, sizeof(size_t), 5, f) == 5;
    ok = ok && std::fwrite(buf.data(), sizeof(float) * 2, (size_t)n, f) == (size_t)n;
    std::fclose(f);
    if (!ok)
        return fail(SMIP_E_RUNTIME, std::string("error writing ") + path);
    return SMIP_OK;
}

// ------------------------------------------------- full stack checkpoint
// bispectrum.dat keeps the reference's format (the normalised bispectrum
// only).  A served job that stops and resumes needs the whole accumulator
// state; this file holds it, after a flush:
//   "SMIPSTK1", int32 W, H, De, dtype, mode, has_ref, int64 nframes, base_size,
//   B, C [base_size] float2, P [hw*H] f64, sum [W*H] 8-byte, shifts [nframes] int2,
//   and for frames: ref frame [W*H] in dtype, ref_sq f64, R [hw*H] float2.
namespace {
bool put(FILE* f, const void* p, size_t n) { return n == 0 || std::fwrite(p, 1, n, f) == n; }
bool get(FILE* f, void* p, size_t n) { return n == 0 || std::fread(p, 1, n, f) == n; }
int dev_to_file(FILE* f, const void* d, size_t n, cudaStream_t st)
{
    std::vector<unsigned char> h(n);
    if (n) {
        CUDA_TRY(cudaMemcpyAsync(h.data(), d, n, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
    }
    return put(f, h.data(), n) ? SMIP_OK : fail(SMIP_E_RUNTIME, "error writing the stack state");
}
int file_to_dev(FILE* f, void* d, size_t n)
{
    std::vector<unsigned char> h(n);
    if (!get(f, h.data(), n))
        return fail(SMIP_E_RUNTIME, "error reading the stack state");
    if (n)
        CUDA_TRY(cudaMemcpy(d, h.data(), n, cudaMemcpyHostToDevice));
    return SMIP_OK;
}
} // namespace

extern "C" int smip_stack_save_state(smip_stack_t s, const char* path)
{
    int rc = smip_stack_sync(s); // flushes the pending batch
    if (rc)
        return rc;
    if (!path)
        return fail(SMIP_E_INVALID_ARGUMENT, "null path");
    FILE* f = std::fopen(path, "wb");
    if (!f)
        return fail(SMIP_E_RUNTIME, std::string("unable to open file ") + path + " for writing");
    const int32_t hdr[6] = { s->g.W, s->g.H, s->g.De, s->dtype, s->mode, s->has_ref ? 1 : 0 };
    const int64_t cnt[2] = { s->nframes, s->g.base_size };
    const size_t bs = (size_t)s->g.base_size, he = s->half_elems(), fe = s->frame_elems();
    bool ok = put(f, "SMIPSTK1", 8) && put(f, hdr, sizeof hdr) && put(f, cnt, sizeof cnt);
    rc = ok ? SMIP_OK : fail(SMIP_E_RUNTIME, "error writing the stack state");
    if (!rc) rc = dev_to_file(f, s->B, sizeof(float2) * bs, s->st);
    if (!rc) rc = dev_to_file(f, s->C, sizeof(float2) * bs, s->st);
    if (!rc) rc = dev_to_file(f, s->P, sizeof(double) * he, s->st);
    if (!rc) rc = dev_to_file(f, s->sum, 8 * fe, s->st);
    if (!rc && s->mode == 1) {
        rc = dev_to_file(f, s->shifts, sizeof(int) * 2 * (size_t)s->nframes, s->st);
        if (!rc) rc = dev_to_file(f, s->ref, dtype_size(s->dtype) * fe, s->st);
        if (!rc) rc = dev_to_file(f, s->ref_sq, sizeof(double), s->st);
        if (!rc) rc = dev_to_file(f, s->R, sizeof(float2) * he, s->st);
    }
    std::fclose(f);
    return rc;
}

extern "C" int smip_stack_load_state(smip_stack_t s, const char* path)
{
    int rc = check_stack(s);
    if (rc)
        return rc;
    if (!path)
        return fail(SMIP_E_INVALID_ARGUMENT, "null path");
    if (s->nframes != 0)
        return fail(SMIP_E_INVALID_ARGUMENT, "stack already holds frames; reset it before loading a state");
    FILE* f = std::fopen(path, "rb");
    if (!f)
        return fail(SMIP_E_RUNTIME, std::string("unable to open file ") + path);
    char magic[8];
    int32_t hdr[6];
    int64_t cnt[2];
    if (!get(f, magic, 8) || std::memcmp(magic, "SMIPSTK1", 8) != 0 || !get(f, hdr, sizeof hdr) || !get(f, cnt, sizeof cnt)) {
        std::fclose(f);
        return fail(SMIP_E_RUNTIME, std::string(path) + ": not a stack state file");
    }
    const int dtype = hdr[3], mode = hdr[4];
    if (hdr[0] != s->g.W || hdr[1] != s->g.H || hdr[2] != s->g.De || cnt[1] != s->g.base_size
        || (mode == 1 && !dtype_size(dtype)) || mode < 0 || mode > 2 || cnt[0] < 0) {
        std::fclose(f);
        return fail(SMIP_E_INVALID_ARGUMENT, std::string("stack state ") + path + " has another shape than the stack");
    }
    const size_t bs = (size_t)s->g.base_size, he = s->half_elems(), fe = s->frame_elems();
    CUDA_TRY(cudaStreamSynchronize(s->st));
    rc = file_to_dev(f, s->B, sizeof(float2) * bs);
    if (!rc) rc = file_to_dev(f, s->C, sizeof(float2) * bs);
    if (!rc) rc = file_to_dev(f, s->P, sizeof(double) * he);
    if (!rc) rc = file_to_dev(f, s->sum, 8 * fe);
    if (!rc && mode == 1) {
        if ((rc = s->ensure_staging(dtype_size(dtype) * fe)) == SMIP_OK)
            s->dtype = dtype;
        if (!rc) rc = s->ensure_shift_cap(cnt[0]);
        if (!rc) rc = file_to_dev(f, s->shifts, sizeof(int) * 2 * (size_t)cnt[0]);
        if (!rc) rc = file_to_dev(f, s->ref, dtype_size(dtype) * fe);
        if (!rc) rc = file_to_dev(f, s->ref_sq, sizeof(double));
        if (!rc) rc = file_to_dev(f, s->R, sizeof(float2) * he);
    }
    std::fclose(f);
    if (rc)
        return rc;
    s->nframes = cnt[0];
    s->pending = 0;
    s->mode = mode;
    s->has_ref = hdr[5] != 0;
    return SMIP_OK;
}

extern "C" int smip_stack_load_bispectrum(smip_stack_t s, const char* path, long nframes)
{
    int rc = check_stack(s);
    if (rc)
        return rc;
    if (!path)
        return fail(SMIP_E_INVALID_ARGUMENT, "null path");
    if (s->nframes != 0)
        return fail(SMIP_E_INVALID_ARGUMENT, "stack already holds frames; reset it before loading a bispectrum");
    FILE* f = std::fopen(path, "rb");
    if (!f)
        return fail(SMIP_E_RUNTIME, std::string("unable to open file ") + path);
    // bispectrum.h:442-461: size_t base_size, 4 x size_t dims, T[base_size]
    size_t hdr[5] = { 0, 0, 0, 0, 0 };
    if (std::fread(hdr, sizeof(size_t), 5, f) != 5) {
        std::fclose(f);
        return fail(SMIP_E_RUNTIME, std::string("error reading bispectrum metadata from file ") + path);
    }
    if (hdr[0] != (size_t)s->g.base_size || hdr[1] != (size_t)s->g.W || hdr[2] != (size_t)s->g.H
        || hdr[3] / 2 * 2 != (size_t)s->g.De || hdr[4] / 2 * 2 != (size_t)s->g.De) {
        std::fclose(f);
        return fail(SMIP_E_INVALID_ARGUMENT, std::string("bispectrum file ") + path + " has another shape than the stack");
    }
    const size_t n = hdr[0];
    std::vector<float> buf(2 * n);
    const bool ok = std::fread(buf.data(), sizeof(float) * 2, n, f) == n;
    std::fclose(f);
    if (!ok)
        return fail(SMIP_E_RUNTIME, std::string("error reading data block from file ") + path);
    return smip_stack_set_bispectrum(s, buf.data(), nframes);
}

extern "C" int smip_stack_set_bispectrum(smip_stack_t s, const float* bispec, long nframes)
{
    int rc = check_stack(s);
    if (rc)
        return rc;
    if (!bispec)
        return fail(SMIP_E_INVALID_ARGUMENT, "null bispectrum");
    if (s->nframes != 0)
        return fail(SMIP_E_INVALID_ARGUMENT, "stack already holds frames; reset it before loading a bispectrum");
    const size_t n = (size_t)s->g.base_size;
    // the normalised bispectrum: the accumulator resumes as it x nframes with
    // zero compensation, over nframes frames
    const long nf = nframes > 0 ? nframes : 1;
    std::vector<float> buf;
    const float* src = bispec;
    if (nf != 1) {
        buf.assign(bispec, bispec + 2 * n);
        for (float& v : buf)
            v = (float)((double)v * (double)nf);
        src = buf.data();
    }
    CUDA_TRY(cudaStreamSynchronize(s->st));
    CUDA_TRY(cudaMemcpy(s->B, src, sizeof(float2) * n, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemset(s->C, 0, sizeof(float2) * n));
    s->nframes = nf;
    s->pending = 0;
    s->mode = 2; // spectra may be added (accumulate_fft); frames need their reference frame
    return SMIP_OK;
}

// ------------------------------------------------------- standalone calls
extern "C" int smip_next_reco_index(double* r, double* phi, int* i, int* j)
{
    if (!r || !phi || !i || !j)
        return fail(SMIP_E_INVALID_ARGUMENT, "null argument");
    next_reco_index(*r, *phi, *i, *j);
    return SMIP_OK;
}

extern "C" int smip_reco_visits(double R, int* ij, long cap, long* count)
{
    std::vector<int2> v = reco_visits(R);
    if (count)
        *count = (long)v.size();
    if (ij)
        for (long q = 0; q < (long)v.size() && q < cap; ++q) {
            ij[2 * q] = v[q].x;
            ij[2 * q + 1] = v[q].y;
        }
    return SMIP_OK;
}

extern "C" int smip_reconstruct_phases(int device, const float* bispec, long xsize, long ysize, long bdepth, double R,
                                       double* phases, unsigned char* flags, double* cons)
{
    Geometry g;
    int rc = make_geometry(xsize, ysize, bdepth, &g);
    if (rc)
        return rc;
    if (!bispec)
        return fail(SMIP_E_INVALID_ARGUMENT, "null bispectrum");
    DeviceCtx* ctx = nullptr;
    if ((rc = device_ctx(device, &ctx)))
        return rc;
    CUDA_TRY(cudaSetDevice(device));
    cudaStream_t st;
    CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    float2* Bd = nullptr;
    int* err = nullptr;
    rc = SMIP_OK;
    {
        Reco reco;
        reco.g = g;
        if (cudaMalloc(&Bd, sizeof(float2) * g.base_size) != cudaSuccess || cudaMalloc(&err, sizeof(int)) != cudaSuccess)
            rc = fail(SMIP_E_NO_MEMORY, "device allocation failed");
        if (!rc && cudaMemcpyAsync(Bd, bispec, sizeof(float2) * g.base_size, cudaMemcpyHostToDevice, st) != cudaSuccess)
            rc = fail(SMIP_E_CUDA, "bispectrum upload failed");
        if (!rc && cudaMemsetAsync(err, 0, sizeof(int), st) != cudaSuccess)
            rc = fail(SMIP_E_CUDA, "memset failed");
        if (!rc)
            rc = reco.run(Bd, R, err, st);
        if (!rc)
            rc = reco.download(phases, flags, cons, st);
        if (!rc)
            rc = check_dev_err(err, st);
        cudaStreamSynchronize(st);
    }
    if (Bd) cudaFree(Bd);
    if (err) cudaFree(err);
    cudaStreamDestroy(st);
    return rc;
}

extern "C" int smip_xcorr_displacement(int device, const double* refimg, const double* frame, long ncols, long nrows,
                                       int* dx, int* dy, double* corr_out)
{
    if (!refimg || !frame || !dx || !dy)
        return fail(SMIP_E_INVALID_ARGUMENT, "null argument");
    smip_stack_t s = nullptr;
    // the smallest depth the shape takes: only the correlation is used
    const long depth = std::max(2L, std::min(8L, (std::min(ncols, nrows) - 1) / 2 * 2));
    int rc = smip_stack_create(&s, device, ncols, nrows, depth, nullptr, 16);
    if (rc)
        return rc;
    const size_t n = (size_t)ncols * nrows;
    std::vector<double> two(2 * n);
    std::memcpy(two.data(), refimg, sizeof(double) * n);
    std::memcpy(two.data() + n, frame, sizeof(double) * n);
    rc = smip_stack_push_frames(s, two.data(), SMIP_F64, 2, 0, 0);
    if (!rc)
        rc = smip_stack_sync(s);
    if (!rc) {
        int xy[2];
        rc = smip_stack_shifts(s, xy, 1, 1);
        *dx = xy[0];
        *dy = xy[1];
        if (!rc && corr_out) {
            // corr of frame 1 of the batch, FP32 -> double
            std::vector<float> c(n);
            if (cudaMemcpy(c.data(), s->corr + n, sizeof(float) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
                rc = fail(SMIP_E_CUDA, "correlation download failed");
            for (size_t i = 0; i < n && !rc; ++i)
                corr_out[i] = c[i];
        }
    }
    smip_stack_destroy(s);
    return rc;
}

extern "C" int smip_bispec_offsets(int device, long ncols, long nrows, long bdepth, const int* idx, long n,
                                   long long* off, int* conj)
{
    // any shape: the index path has no size restriction of its own
    if (ncols < 1 || nrows < 1 || bdepth < 0 || ncols > (1 << 20) || nrows > (1 << 20) || bdepth > (1 << 20))
        return fail(SMIP_E_INVALID_ARGUMENT, "invalid bispectrum extents");
    Geometry g {};
    g.W = (int)ncols;
    g.H = (int)nrows;
    g.De = (int)(bdepth / 2) * 2;
    if (n < 0 || (n > 0 && (!idx || !off || !conj)))
        return fail(SMIP_E_INVALID_ARGUMENT, "invalid buffers");
    if (n == 0)
        return SMIP_OK;
    CUDA_TRY(cudaSetDevice(device));
    int* di = nullptr;
    long long* doff = nullptr;
    int* dc = nullptr;
    cudaError_t e = cudaMalloc(&di, sizeof(int) * 4 * n);
    if (e == cudaSuccess) e = cudaMalloc(&doff, sizeof(long long) * n);
    if (e == cudaSuccess) e = cudaMalloc(&dc, sizeof(int) * n);
    if (e == cudaSuccess) e = cudaMemcpy(di, idx, sizeof(int) * 4 * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = launch_offset_probe(g, di, n, doff, dc, 0);
    if (e == cudaSuccess) e = cudaMemcpy(off, doff, sizeof(long long) * n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(conj, dc, sizeof(int) * n, cudaMemcpyDeviceToHost);
    if (di) cudaFree(di);
    if (doff) cudaFree(doff);
    if (dc) cudaFree(dc);
    if (e != cudaSuccess)
        return fail(SMIP_E_CUDA, cudaGetErrorString(e));
    return SMIP_OK;
}

extern "C" int smip_shifted(int device, const double* in, double* out, long ncols, long nrows, int dx, int dy)
{
    if (!in || !out)
        return fail(SMIP_E_INVALID_ARGUMENT, "null array");
    if (ncols <= 0 || nrows <= 0 || ncols * nrows > (1L << 30))
        return fail(SMIP_E_INVALID_ARGUMENT, "invalid array size");
    // the reference's clamped range reads outside the array for |distance| >= size
    if (dx <= -ncols || dx >= ncols || dy <= -nrows || dy >= nrows)
        return fail(SMIP_E_OUT_OF_RANGE, "Array2::shifted: distance not smaller than the array size");
    CUDA_TRY(cudaSetDevice(device));
    const size_t bytes = sizeof(double) * (size_t)(ncols * nrows);
    double *din = nullptr, *dout = nullptr;
    CUDA_TRY(cudaMalloc(&din, bytes));
    cudaError_t e = cudaMalloc(&dout, bytes);
    if (e == cudaSuccess)
        e = cudaMemcpy(din, in, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = launch_shifted(din, dout, (int)ncols, (int)nrows, dx, dy, 0);
    if (e == cudaSuccess)
        e = cudaMemcpy(out, dout, bytes, cudaMemcpyDeviceToHost);
    cudaFree(din);
    if (dout)
        cudaFree(dout);
    if (e != cudaSuccess)
        return fail(SMIP_E_CUDA, cudaGetErrorString(e));
    return SMIP_OK;
}

extern "C" int smip_hann(int device, double* out, long xsize, long ysize, double aperture)
{
    if (!out)
        return fail(SMIP_E_INVALID_ARGUMENT, "null output");
    if (!(aperture > 0.))
        return fail(SMIP_E_DOMAIN, "WindowFunction aperture size <= 0");
    if (xsize < 1 || ysize < 1)
        return fail(SMIP_E_INVALID_ARGUMENT, "window size must be positive");
    CUDA_TRY(cudaSetDevice(device));
    double* d = nullptr;
    CUDA_TRY(cudaMalloc(&d, sizeof(double) * xsize * ysize));
    cudaError_t e = launch_hann(d, (int)xsize, (int)ysize, aperture, 0);
    if (e == cudaSuccess)
        e = cudaMemcpy(out, d, sizeof(double) * xsize * ysize, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess)
        return fail(SMIP_E_CUDA, cudaGetErrorString(e));
    return SMIP_OK;
}
