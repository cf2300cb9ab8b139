// mcig_capi.cu -- the C ABI of include/mcig.h: host orchestration of MCI::integrate
// (reference src/MCIntegrator.cpp:43-82) over the device kernels.
//
// Compiled with -fmad=false: the estimator kernels in this unit follow the
// reference's double operation order.
#include <cuda_runtime.h>
#include <dlfcn.h>

#include <algorithm>
#include <chrono>
#include <fstream>
#include <numeric>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <map>
#include <vector>

#include "../../include/mcig.h"
#include "mcig_common.cuh"
#include "mcig_estimators.cuh"
#include "mcig_generic.cuh"
#include "mcig_launchers.h"
#include "mcig_batch.h"

// ------------------------------------------------------------------------
// errors
// ------------------------------------------------------------------------
static thread_local std::string g_err;

static int set_err(int code, const char *fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) { return set_err(MCIG_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); } \
    } while (0)

extern "C" const char *mcig_last_error(void) { return g_err.c_str(); }

// error setter for the other translation units of the library
int mcig_set_last_error(int code, const char *msg)
{
    g_err = msg ? msg : "";
    return code;
}
extern "C" const char *mcig_version(void) { return "mcig 0.1 (sm_103a)"; }

// ------------------------------------------------------------------------
// device buffer helper
// ------------------------------------------------------------------------
template <class T> struct DBuf {
    T *p = nullptr;
    size_t n = 0;
    int alloc(size_t count)
    {
        if (count <= n && p) { return MCIG_OK; }
        release();
        if (count == 0) { return MCIG_OK; }
        cudaError_t e = cudaMalloc((void **)&p, count * sizeof(T));
        if (e != cudaSuccess) { p = nullptr; n = 0; return set_err(MCIG_ERR_CUDA, "cudaMalloc(%zu bytes): %s", count * sizeof(T), cudaGetErrorString(e)); }
        n = count;
        return MCIG_OK;
    }
    void release()
    {
        if (p) { cudaFree(p); }
        p = nullptr;
        n = 0;
    }
};

struct PdfDef {
    int kind;
    std::vector<double> params;
};

struct ObsDef {
    int kind;
    std::vector<double> params;
    int nv, blocksize, nskip, flag_equil, estimator, acc;
};

// a loaded plugin (include/mcig/plugin.cuh): its user functors and its general kernel
struct mcig_plugin {
    void *dl = nullptr;
    int npdf = 0, nobs = 0, nmove = 0;
    int (*pdf_nproto)(int, int) = nullptr;
    int (*obs_nvals)(int, int) = nullptr;
    mcig_plugin_launch_fn (*launcher)(int, int) = nullptr;
    // trial moves (optional exports of MCIG_PLUGIN_MOVES)
    int (*move_info)(int, int, const double *, int, int *, int *, double *) = nullptr;
    int (*move_steps)(int, int, const double *, int, int, double *, int *) = nullptr;
};

#define MCIG_MAX_CHUNKS 8

struct mcig_mci {
    int ndim;
    const mcig_plugin *plugin = nullptr; // user functors (MCIG_PDF_USER / MCIG_OBS_USER kinds)
    int64_t nchains;
    int device;
    int prec;
    cudaStream_t stream = nullptr;
    uint64_t seed = 0;
    // trial move
    int movetype = MCIG_MOVE_ALL, srrd = MCIG_SRRD_UNIFORM, veclen = 0, ntypes = 1;
    int typeEnds[MCIG_MAXTYPES] = {0, 0, 0, 0};
    int ms_nsteps = 0, ms_srrd = 0, ms_veclen = 1;
    // user trial move (MCIG_MOVE_USER): plugin move index, parameters, proto values, the step
    // size index of every coordinate (getStepSizeIndex)
    int umove = 0, umove_nproto = 0;
    std::vector<double> umove_params;
    std::vector<int> umove_stepidx;
    std::vector<PdfDef> ms_pdfs, pdfs;
    std::vector<ObsDef> obs;
    int periodic = 0;
    std::vector<double> lb, ub;
    // file output of the main sampling (MCI::storeObservablesOnFile / storeWalkerPositionsOnFile)
    std::string obs_path, wlk_path;
    int obs_freq = 0, wlk_freq = 0;
    DBuf<int64_t> dump_steps;
    DBuf<double> dump_x, dump_vals;
    double target = 0.5;
    int nfind = -50;
    int64_t ndecorr = -10000;
    int full32 = 0;
    int kernel_policy = 0; // 0 auto, 1 general kernel, 2 register-resident kernel
    int fuse_phases = 0;   // 1: calibration, burn-in and sampling in one register-resident launch
    int calib_split = 1;   // calibration's tail split over lanes where mcig_calib.cuh serves it
    int lanes = 0;         // lanes per chain of the multi-lane mixture kernel (0: one lane per chain)
    int f64_decide = 0;    // Metropolis decision certified in double (multi-lane kernel): 0 off, 1, 2
    DBuf<unsigned long long> dstats; // [checked, reversed, largest reversed float margin (float bits)]
    FastConst fc;          // constant data of the register-resident kernel
    // device chain state
    DBuf<double> x, step;
    DBuf<uint64_t> ctr;
    DBuf<int64_t> tpos, nacc, nrej, tape_len;
    DBuf<int> status;
    DBuf<double> params, lbub, stepmax, xstage;
    DBuf<float> fblob;
    DBuf<double> tape;
    int64_t tape_stride = 0;
    bool replay = false;
    // observable data of the last integrate
    std::vector<DBuf<char>> obsdata;
    std::vector<int64_t> obs_nstore;
    DBuf<double> est_avg, est_err, scratch;
    DBuf<uint8_t> active;
    // results.  After an integrate the per-chain estimates (est_avg/est_err, scaled by
    // chain_scale) and the counts stay on the device; the host copies are made when
    // asked for (host_results()).
    mutable std::vector<double> chain_avg, chain_err;
    mutable std::vector<int64_t> h_nacc, h_nrej;
    mutable bool chains_on_device = false, counts_on_device = false;
    double chain_scale = 1.;
    DBuf<double> comb;      // combined average[nod], error[nod]
    double *h_comb = nullptr; // pinned staging of comb
    bool record = false;
    DBuf<uint8_t> bits;
    int64_t bits_steps = 0;
    double ms[4] = {0, 0, 0, 0};
    int64_t launches = 0;
    cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    // chunked sampling (mcig_set_sampling_chunks): the Uncorrelated estimator of float Full
    // samples runs on a low-priority stream over each finished chunk beside the next one;
    // off by default (at 65,536 chains of the 16-D workload the sampling kernel holds the
    // SMs' registers and the estimator ran mostly after it: 10.9 ms of estimation tail
    // against 8.1 ms for the one-pass estimator)
    int chunks = 1;
    cudaStream_t est_stream = nullptr;
    cudaEvent_t cev[MCIG_MAX_CHUNKS + 1] = {};
    DBuf<float4> est_state;
};

static int nobsdim(const mcig_mci *h)
{
    int n = 0;
    for (auto &o : h->obs) { n += o.nv; }
    return n;
}

static int maxd_bucket(int ndim)
{
    const int b[] = {4, 8, 16, 32, 64};
    for (int v : b) {
        if (ndim <= v) { return v; }
    }
    return 0;
}

// ------------------------------------------------------------------------
// validation of functor parameters (mirrors the oracle's pdf_init / obs_init)
// ------------------------------------------------------------------------
static int check_pdf(int ndim, int kind, const double *params, int np)
{
    switch (kind) {
    case MCIG_PDF_GAUSS_SUM:
    case MCIG_PDF_GAUSS:
    case MCIG_PDF_EXP: return MCIG_OK;
    case MCIG_PDF_GAUSS_PREC:
        if (np != ndim * ndim) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "GAUSS_PREC needs ndim*ndim params"); }
        return MCIG_OK;
    case MCIG_PDF_GAUSS_BLOCK:
        if (np != 3) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "GAUSS_BLOCK needs [b0,b1,w]"); }
        if ((int)params[0] < 0 || (int)params[1] > ndim || (int)params[0] >= (int)params[1] || !(params[2] > 0.)) {
            return set_err(MCIG_ERR_INVALID_ARGUMENT, "GAUSS_BLOCK bad block");
        }
        return MCIG_OK;
    case MCIG_PDF_GAUSS_MIX: {
        if (np < 1) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "GAUSS_MIX needs params"); }
        const int nc = (int)params[0];
        if (nc < 1 || nc > 16 || np != 1 + nc + 2 * nc * ndim) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "GAUSS_MIX bad param count (1..16 components)"); }
        return MCIG_OK;
    }
    default: return set_err(MCIG_ERR_INVALID_ARGUMENT, "unknown sampling function kind %d", kind);
    }
}

static int obs_nvals(int ndim, int kind, const double *params, int np, int *nv)
{
    switch (kind) {
    case MCIG_OBS_X2SUM:
    case MCIG_OBS_X2MEAN:
    case MCIG_OBS_POLYNOM:
    case MCIG_OBS_GAUSSX2:
    case MCIG_OBS_LOGPDF: *nv = 1; return MCIG_OK;
    case MCIG_OBS_CONST:
        if (np < 1) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "CONST needs its value"); }
        *nv = 1;
        return MCIG_OK;
    case MCIG_OBS_XND:
    case MCIG_OBS_X2: *nv = ndim; return MCIG_OK;
    case MCIG_OBS_XI:
        if (np < 1 || (int)params[0] < 0 || (int)params[0] >= ndim) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "XI needs an index in [0, ndim)"); }
        *nv = 1;
        return MCIG_OK;
    case MCIG_OBS_X2BLOCK: {
        if (np < 2) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "X2BLOCK needs [nb, b0..b_nb]"); }
        const int nb = (int)params[0];
        if (nb < 1 || np != nb + 2) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "X2BLOCK bad param count"); }
        for (int k = 0; k < nb; ++k) {
            if ((int)params[1 + k] < 0 || (int)params[2 + k] > ndim || (int)params[1 + k] > (int)params[2 + k]) {
                return set_err(MCIG_ERR_INVALID_ARGUMENT, "X2BLOCK bad bounds");
            }
        }
        *nv = nb;
        return MCIG_OK;
    }
    default: return set_err(MCIG_ERR_INVALID_ARGUMENT, "unknown observable kind %d", kind);
    }
}

// plugin kinds (include/mcig/plugin.cuh): the k-th functor of the attached plugin
static bool is_user_pdf(int kind) { return kind >= MCIG_PDF_USER; }
static bool is_user_obs(int kind) { return kind >= MCIG_OBS_USER; }

static int user_pdf_nproto(const mcig_mci *h, int kind, int *nproto)
{
    if (!h->plugin) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "sampling function kind %d is a plugin kind and the handle has no plugin", kind); }
    const int k = kind - MCIG_PDF_USER;
    if (k >= h->plugin->npdf) {
        return set_err(MCIG_ERR_INVALID_ARGUMENT, "the plugin has %d sampling functions, kind %d asks for number %d", h->plugin->npdf, kind, k);
    }
    const int n = h->plugin->pdf_nproto(k, h->ndim);
    if (n < 0) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "plugin sampling function %d: nproto(%d) is above its max_nproto", k, h->ndim); }
    *nproto = n;
    return MCIG_OK;
}

static int user_obs_nvals(const mcig_mci *h, int kind, int *nv)
{
    if (!h->plugin) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "observable kind %d is a plugin kind and the handle has no plugin", kind); }
    const int k = kind - MCIG_OBS_USER;
    if (k >= h->plugin->nobs) {
        return set_err(MCIG_ERR_INVALID_ARGUMENT, "the plugin has %d observables, kind %d asks for number %d", h->plugin->nobs, kind, k);
    }
    const int n = h->plugin->obs_nvals(k, h->ndim);
    if (n < 1) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "plugin observable %d: nobs(%d) = %d", k, h->ndim, n); }
    *nv = n;
    return MCIG_OK;
}

static bool uses_plugin(const mcig_mci *h)
{
    for (auto &d : h->pdfs) {
        if (is_user_pdf(d.kind)) { return true; }
    }
    for (auto &d : h->ms_pdfs) {
        if (is_user_pdf(d.kind)) { return true; }
    }
    for (auto &o : h->obs) {
        if (is_user_obs(o.kind)) { return true; }
    }
    return h->movetype == MCIG_MOVE_USER;
}

// what the plugin kernel does not serve
static int check_plugin_use(const mcig_mci *h)
{
    if (!uses_plugin(h)) { return MCIG_OK; }
    if (!h->plugin) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "plugin kinds are in use and the handle has no plugin"); }
    bool upd = false, uob = false;
    for (auto &d : h->pdfs) { upd = upd || is_user_pdf(d.kind); }
    for (auto &o : h->obs) { uob = uob || is_user_obs(o.kind); }
    for (auto &o : h->obs) {
        if (upd && o.kind == MCIG_OBS_LOGPDF) { return set_err(MCIG_ERR_UNSUPPORTED, "the LOGPDF observable reads built-in sampling functions only"); }
    }
    if (uob && h->obs_freq > 0) { return set_err(MCIG_ERR_UNSUPPORTED, "observable file output is not served for plugin observables"); }
    return MCIG_OK;
}

// ------------------------------------------------------------------------
// creation / state
// ------------------------------------------------------------------------
static int upload_state_defaults(mcig_mci *h)
{
    const size_t nc = (size_t)h->nchains;
    int rc;
    if ((rc = h->x.alloc(nc * h->ndim)) || (rc = h->step.alloc(nc * MCIG_MAXTYPES)) || (rc = h->ctr.alloc(nc)) ||
        (rc = h->tpos.alloc(nc)) || (rc = h->nacc.alloc(nc)) || (rc = h->nrej.alloc(nc)) || (rc = h->status.alloc(1))) {
        return rc;
    }
    CK(cudaMemsetAsync(h->x.p, 0, nc * h->ndim * sizeof(double), h->stream));
    CK(cudaMemsetAsync(h->ctr.p, 0, nc * sizeof(uint64_t), h->stream));
    CK(cudaMemsetAsync(h->tpos.p, 0, nc * sizeof(int64_t), h->stream));
    CK(cudaMemsetAsync(h->nacc.p, 0, nc * sizeof(int64_t), h->stream));
    CK(cudaMemsetAsync(h->nrej.p, 0, nc * sizeof(int64_t), h->stream));
    return MCIG_OK;
}

static int fill_steps(mcig_mci *h, double v)
{
    std::vector<double> s((size_t)h->nchains * MCIG_MAXTYPES, v);
    CK(cudaMemcpyAsync(h->step.p, s.data(), s.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return MCIG_OK;
}

extern "C" int mcig_create(int ndim, int64_t nchains, int device, int precision, mcig_mci **out)
{
    if (!out) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "out is NULL"); }
    *out = nullptr;
    if (ndim < 1) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "[ProtoFunctionInterface] Number of dimensions must be at least 1."); }
    if (maxd_bucket(ndim) == 0) { return set_err(MCIG_ERR_UNSUPPORTED, "ndim %d exceeds the device maximum of 64", ndim); }
    if (nchains < 1 || nchains > (int64_t)1 << 30) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "nchains must be in [1, 2^30]"); }
    if (precision < MCIG_PREC_FP64 || precision > MCIG_PREC_FP32_ACC64) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "bad precision"); }
    int ndev = 0;
    CK(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "device %d not present (%d devices)", device, ndev); }
    CK(cudaSetDevice(device));
    mcig_mci *h = new mcig_mci();
    h->ndim = ndim;
    h->nchains = nchains;
    h->device = device;
    h->prec = precision;
    h->typeEnds[0] = ndim;
    int prio_low = 0, prio_high = 0; // the handle's stream gets the highest priority, so that the
    cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high); // chunk estimators never hold back sampling
    cudaError_t e = cudaStreamCreateWithPriority(&h->stream, cudaStreamNonBlocking, prio_high);
    if (e != cudaSuccess) {
        delete h;
        return set_err(MCIG_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
    }
    for (auto &ev : h->ev) { cudaEventCreate(&ev); }
    int rc = upload_state_defaults(h);
    if (!rc) { rc = fill_steps(h, 0.05); } // DEFAULT_MRT2STEP (Factories.hpp:145)
    if (rc) {
        mcig_destroy(h);
        return rc;
    }
    *out = h;
    return MCIG_OK;
}

// ------------------------------------------------------------------------
// plugins (include/mcig/plugin.cuh)
// ------------------------------------------------------------------------
extern "C" int mcig_plugin_load(const char *path, mcig_plugin **out)
{
    if (!path || !out) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "path or out is NULL"); }
    *out = nullptr;
    void *dl = dlopen(path, RTLD_NOW | RTLD_LOCAL);
    if (!dl) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "plugin %s: %s", path, dlerror()); }
    auto sym = [&](const char *name) { return dlsym(dl, name); };
    auto abi = (int (*)(void))sym("mcig_plugin_abi");
    auto kps = (int (*)(void))sym("mcig_plugin_kparams_size");
    auto npdf = (int (*)(void))sym("mcig_plugin_npdf");
    auto nobs = (int (*)(void))sym("mcig_plugin_nobs");
    auto pl = new mcig_plugin;
    pl->pdf_nproto = (int (*)(int, int))sym("mcig_plugin_pdf_nproto");
    pl->obs_nvals = (int (*)(int, int))sym("mcig_plugin_obs_nvals");
    pl->launcher = (mcig_plugin_launch_fn(*)(int, int))sym("mcig_plugin_launcher");
    if (!abi || !kps || !npdf || !nobs || !pl->pdf_nproto || !pl->obs_nvals || !pl->launcher) {
        delete pl;
        dlclose(dl);
        return set_err(MCIG_ERR_INVALID_ARGUMENT, "plugin %s does not export the plugin entry points (MCIG_PLUGIN)", path);
    }
    if (abi() != MCIG_PLUGIN_ABI || kps() != (int)sizeof(KParams)) {
        delete pl;
        dlclose(dl);
        return set_err(MCIG_ERR_INVALID_ARGUMENT, "plugin %s was built against another version of the integrator", path);
    }
    pl->npdf = npdf();
    pl->nobs = nobs();
    auto nmove = (int (*)(void))sym("mcig_plugin_nmove");
    pl->move_info = (int (*)(int, int, const double *, int, int *, int *, double *))sym("mcig_plugin_move_info");
    pl->move_steps = (int (*)(int, int, const double *, int, int, double *, int *))sym("mcig_plugin_move_steps");
    pl->nmove = (nmove && pl->move_info && pl->move_steps) ? nmove() : 0;
    if (pl->npdf > MCIG_MAXUSER || pl->nobs > MCIG_MAXUSER) {
        delete pl;
        dlclose(dl);
        return set_err(MCIG_ERR_UNSUPPORTED, "plugin %s: at most %d sampling functions and %d observables", path, MCIG_MAXUSER, MCIG_MAXUSER);
    }
    pl->dl = dl;
    *out = pl;
    return MCIG_OK;
}

extern "C" int mcig_plugin_unload(mcig_plugin *pl)
{
    if (!pl) { return MCIG_OK; }
    if (pl->dl) { dlclose(pl->dl); }
    delete pl;
    return MCIG_OK;
}

extern "C" int mcig_plugin_counts(const mcig_plugin *pl, int *npdf, int *nobs)
{
    if (!pl) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "plugin is NULL"); }
    if (npdf) { *npdf = pl->npdf; }
    if (nobs) { *nobs = pl->nobs; }
    return MCIG_OK;
}

extern "C" int mcig_plugin_nmoves(const mcig_plugin *pl, int *nmove)
{
    if (!pl || !nmove) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "plugin or nmove is NULL"); }
    *nmove = pl->nmove;
    return MCIG_OK;
}

extern "C" int mcig_set_plugin(mcig_mci *h, const mcig_plugin *pl)
{
    if (!h) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "handle is NULL"); }
    if (!pl && uses_plugin(h)) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "the handle holds plugin kinds: remove them before detaching the plugin"); }
    if (pl && h->plugin && pl != h->plugin && uses_plugin(h)) {
        return set_err(MCIG_ERR_INVALID_ARGUMENT, "the handle holds kinds of another plugin: remove them first");
    }
    h->plugin = pl;
    return MCIG_OK;
}

extern "C" int mcig_destroy(mcig_mci *h)
{
    if (!h) { return MCIG_OK; }
    cudaSetDevice(h->device);
    if (h->stream) { cudaStreamSynchronize(h->stream); }
    h->x.release(); h->step.release(); h->ctr.release(); h->tpos.release(); h->nacc.release(); h->nrej.release();
    h->tape_len.release(); h->status.release(); h->params.release(); h->lbub.release(); h->stepmax.release();
    h->fblob.release(); h->tape.release(); h->est_avg.release(); h->est_err.release(); h->scratch.release();
    h->comb.release();
    h->xstage.release();
    h->dump_steps.release(); h->dump_x.release(); h->dump_vals.release();
    if (h->h_comb) { cudaFreeHost(h->h_comb); h->h_comb = nullptr; }
    h->active.release(); h->bits.release();
    for (auto &b : h->obsdata) { b.release(); }
    for (auto &ev : h->ev) { if (ev) { cudaEventDestroy(ev); } }
    for (auto &ev : h->cev) { if (ev) { cudaEventDestroy(ev); } }
    h->est_state.release(); h->dstats.release();
    if (h->est_stream) { cudaStreamSynchronize(h->est_stream); cudaStreamDestroy(h->est_stream); }
    if (h->stream) { cudaStreamDestroy(h->stream); }
    delete h;
    return MCIG_OK;
}

extern "C" int mcig_get_ndim(const mcig_mci *h, int *ndim) { *ndim = h->ndim; return MCIG_OK; }
extern "C" int64_t mcig_get_nchains(const mcig_mci *h) { return h->nchains; }
extern "C" void *mcig_get_stream(const mcig_mci *h) { return (void *)h->stream; }

extern "C" int mcig_set_precision(mcig_mci *h, int precision)
{
    if (precision < MCIG_PREC_FP64 || precision > MCIG_PREC_FP32_ACC64) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "bad precision"); }
    if (h->replay && precision != MCIG_PREC_FP64) { return set_err(MCIG_ERR_UNSUPPORTED, "replay needs MCIG_PREC_FP64"); }
    h->prec = precision;
    return MCIG_OK;
}

extern "C" int mcig_set_seed(mcig_mci *h, uint64_t seed)
{
    h->seed = seed;
    cudaSetDevice(h->device);
    CK(cudaMemsetAsync(h->ctr.p, 0, (size_t)h->nchains * sizeof(uint64_t), h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return MCIG_OK;
}

static void apply_domain_host(const mcig_mci *h, double *x)
{
    if (!h->periodic) { return; }
    for (int i = 0; i < h->ndim; ++i) {
        while (x[i] < h->lb[i]) { x[i] += h->ub[i] - h->lb[i]; }
        while (x[i] > h->ub[i]) { x[i] -= h->ub[i] - h->lb[i]; }
    }
}

// rows x[n][ndim] (n == 1: one row for every chain) -> walkers [ndim][nchains]
static __global__ void rows_to_walkers_kernel(const double *__restrict__ rows, int64_t n, int ndim, int64_t nc, double *x)
{
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= nc) { return; }
    const double *src = rows + (n == 1 ? 0 : c * ndim);
    for (int i = 0; i < ndim; ++i) { x[(size_t)i * nc + c] = src[i]; }
}

extern "C" int mcig_set_x(mcig_mci *h, const double *x, int64_t n)
{
    if (!x) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "x is NULL"); }
    if (n != 1 && n != h->nchains) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "set_x: n must be 1 or nchains"); }
    cudaSetDevice(h->device);
    if (!h->periodic) { // the unbound domain leaves x as it is: copy the rows and transpose on the device
        int rc;
        if ((rc = h->xstage.alloc((size_t)n * h->ndim))) { return rc; }
        CK(cudaMemcpyAsync(h->xstage.p, x, (size_t)n * h->ndim * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        rows_to_walkers_kernel<<<(int)((h->nchains + 255) / 256), 256, 0, h->stream>>>(h->xstage.p, n, h->ndim, h->nchains, h->x.p);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(h->stream)); // the caller may reuse x on return
        return MCIG_OK;
    }
    const size_t nc = (size_t)h->nchains;
    std::vector<double> t(nc * h->ndim);
    std::vector<double> v(h->ndim);
    for (size_t c = 0; c < nc; ++c) {
        const double *src = x + (n == 1 ? 0 : c * h->ndim);
        std::copy(src, src + h->ndim, v.begin());
        apply_domain_host(h, v.data()); // MCI::setX applies the domain (MCIntegrator.cpp:594-604)
        for (int i = 0; i < h->ndim; ++i) { t[(size_t)i * nc + c] = v[i]; }
    }
    CK(cudaMemcpyAsync(h->x.p, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return MCIG_OK;
}

extern "C" int mcig_get_x(mcig_mci *h, double *x)
{
    cudaSetDevice(h->device);
    const size_t nc = (size_t)h->nchains;
    std::vector<double> t(nc * h->ndim);
    CK(cudaMemcpyAsync(t.data(), h->x.p, t.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (size_t c = 0; c < nc; ++c) {
        for (int i = 0; i < h->ndim; ++i) { x[c * h->ndim + i] = t[(size_t)i * nc + c]; }
    }
    return MCIG_OK;
}

extern "C" int mcig_center_x(mcig_mci *h)
{
    std::vector<double> v(h->ndim, 0.);
    if (h->periodic) { // DomainInterface::getCenter (DomainInterface.hpp:36-40)
        for (int i = 0; i < h->ndim; ++i) { v[i] = h->lb[i] + 0.5 * (h->ub[i] - h->lb[i]); }
    }
    return mcig_set_x(h, v.data(), 1);
}

static int nstepsizes(const mcig_mci *h) { return h->ntypes; }

extern "C" int mcig_set_mrt2step(mcig_mci *h, double v)
{
    cudaSetDevice(h->device);
    return fill_steps(h, v);
}

extern "C" int mcig_set_mrt2step_i(mcig_mci *h, int i, double v)
{
    if (i < 0 || i >= nstepsizes(h)) {
        std::printf("[MCI::setMRT2Step] Warning: Tried to set non-existing MRT2step index.\n");
        return MCIG_OK;
    }
    cudaSetDevice(h->device);
    std::vector<double> s((size_t)h->nchains, v);
    CK(cudaMemcpyAsync(h->step.p + (size_t)i * h->nchains, s.data(), s.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return MCIG_OK;
}

extern "C" int mcig_get_nstepsizes(const mcig_mci *h, int *n) { *n = nstepsizes(h); return MCIG_OK; }

extern "C" int mcig_get_mrt2step(const mcig_mci *h, int64_t chain, int i, double *v)
{
    if (chain < 0 || chain >= h->nchains) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "chain out of range"); }
    if (i < 0 || i >= nstepsizes(h)) { *v = 0.; return MCIG_OK; }
    cudaSetDevice(h->device);
    CK(cudaMemcpyAsync(v, h->step.p + (size_t)i * h->nchains + chain, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return MCIG_OK;
}

extern "C" int mcig_get_mrt2steps(const mcig_mci *h, double *steps)
{
    cudaSetDevice(h->device);
    const size_t nc = (size_t)h->nchains;
    const int ns = nstepsizes(h);
    std::vector<double> t(nc * ns);
    CK(cudaMemcpyAsync(t.data(), h->step.p, t.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (size_t c = 0; c < nc; ++c) {
        for (int i = 0; i < ns; ++i) { steps[c * ns + i] = t[(size_t)i * nc + c]; }
    }
    return MCIG_OK;
}

extern "C" int mcig_set_target_acceptance_rate(mcig_mci *h, double r) { h->target = r; return MCIG_OK; }
extern "C" int mcig_set_nfind_mrt2_iterations(mcig_mci *h, int n) { h->nfind = n; return MCIG_OK; }
extern "C" int mcig_set_ndecorrelation_steps(mcig_mci *h, int64_t n) { h->ndecorr = n; return MCIG_OK; }

extern "C" int mcig_set_multistep_move(mcig_mci *h, int nsteps, int sub_srrd, int sub_veclen, double sub_step)
{
    if (sub_srrd < MCIG_SRRD_UNIFORM || sub_srrd > MCIG_SRRD_FISHER) { return set_err(MCIG_ERR_DOMAIN, "[createSRRDVecMove] Unhandled SRRDType enumerator."); }
    if (sub_veclen < 1 || h->ndim % sub_veclen != 0) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "[MCI::setTrialMove] MCI's number of walkers must be a multiple of passed veclen."); }
    if (nsteps < 0 || nsteps > 65534) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "multi-step move: nsteps must be in [0, 65534]"); }
    h->movetype = MCIG_MOVE_MULTISTEP;
    h->ms_nsteps = nsteps;
    h->ms_srrd = sub_srrd;
    h->ms_veclen = sub_veclen;
    h->ms_pdfs.clear();
    h->ntypes = 1;
    h->typeEnds[0] = h->ndim;
    cudaSetDevice(h->device);
    return fill_steps(h, sub_step);
}

extern "C" int mcig_set_trial_move(mcig_mci *h, int movetype, int srrd, int veclen, int ntypes, const int *typeEnds)
{
    if (movetype == MCIG_MOVE_MULTISTEP) { return mcig_set_multistep_move(h, h->ndim, MCIG_SRRD_UNIFORM, 1, 0.05); }
    if (movetype != MCIG_MOVE_ALL && movetype != MCIG_MOVE_VEC) { return set_err(MCIG_ERR_DOMAIN, "[createMoveDefault] Unhandled MoveType enumerator."); }
    if (srrd < MCIG_SRRD_UNIFORM || srrd > MCIG_SRRD_FISHER) { return set_err(MCIG_ERR_DOMAIN, "[createSRRDAllMove] Unhandled SRRDType enumerator."); }
    if (ntypes < 1) { ntypes = 1; }
    if (ntypes > MCIG_MAXTYPES) { return set_err(MCIG_ERR_UNSUPPORTED, "at most %d step-size types on the device", MCIG_MAXTYPES); }
    const int vl = (movetype == MCIG_MOVE_VEC) ? std::max(1, veclen) : 0;
    if (vl > 0 && h->ndim % vl != 0) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "[MCI::setTrialMove] MCI's number of walkers must be a multiple of passed veclen."); }
    if (ntypes > 1 && !typeEnds) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "[TypedMoveInterface] When ntypes>1, passed typeEnds must not be null."); }
    if (ntypes > 1 && vl > 0) {
        for (int i = 0; i < ntypes; ++i) {
            if (typeEnds[i] % vl != 0) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "[SRRDVecMove] All type end indices must be multiples of vector length."); }
        }
    }
    h->movetype = (vl > 0) ? MCIG_MOVE_VEC : MCIG_MOVE_ALL;
    h->srrd = srrd;
    h->veclen = vl;
    h->ntypes = ntypes;
    for (int i = 0; i < MCIG_MAXTYPES; ++i) { h->typeEnds[i] = (ntypes > 1 && i < ntypes) ? typeEnds[i] : h->ndim; }
    cudaSetDevice(h->device);
    return fill_steps(h, 0.05);
}

extern "C" int mcig_set_user_move(mcig_mci *h, int k, const double *params, int nparams)
{
    if (!h) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "handle is NULL"); }
    if (!h->plugin) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "a user trial move needs a plugin: the handle has no plugin"); }
    if (k < 0 || k >= h->plugin->nmove) {
        return set_err(MCIG_ERR_INVALID_ARGUMENT, "the plugin has %d trial moves, not a move %d", h->plugin->nmove, k);
    }
    if (nparams < 0 || (nparams > 0 && !params)) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "move parameters"); }
    const std::vector<double> par(params, params + nparams);
    int nproto = 0, nstep = 0;
    double rate = 0.;
    if (h->plugin->move_info(k, h->ndim, par.data(), nparams, &nproto, &nstep, &rate) != 0 || nproto < 0) {
        return set_err(MCIG_ERR_INVALID_ARGUMENT, "trial move %d: nproto(%d) is above its max_nproto", k, h->ndim);
    }
    if (nstep < 0 || nstep > MCIG_MAXTYPES) {
        return set_err(MCIG_ERR_UNSUPPORTED, "trial move %d has %d step sizes; at most %d on the device", k, nstep, MCIG_MAXTYPES);
    }
    std::vector<double> s0(std::max(nstep, 1), 0.);
    std::vector<int> idx(h->ndim, 0);
    h->plugin->move_steps(k, h->ndim, par.data(), nparams, nstep, s0.data(), idx.data());
    for (int i = 0; i < h->ndim && nstep > 0; ++i) {
        if (idx[i] < 0 || idx[i] >= nstep) {
            return set_err(MCIG_ERR_INVALID_ARGUMENT, "trial move %d: step size index %d of coordinate %d is not in [0, %d)", k, idx[i], i, nstep);
        }
    }
    h->movetype = MCIG_MOVE_USER;
    h->umove = k;
    h->umove_nproto = nproto;
    h->umove_params = par;
    h->umove_stepidx = idx;
    h->ms_pdfs.clear();
    h->ntypes = nstep;
    for (int i = 0; i < MCIG_MAXTYPES; ++i) { h->typeEnds[i] = h->ndim; }
    cudaSetDevice(h->device);
    if (nstep == 0) { return MCIG_OK; }
    int rc = fill_steps(h, s0[0]);
    for (int t = 1; t < nstep && rc == MCIG_OK; ++t) { rc = mcig_set_mrt2step_i(h, t, s0[t]); }
    return rc;
}

extern "C" int mcig_multistep_add_pdf(mcig_mci *h, int kind, const double *params, int nparams)
{
    if (h->movetype != MCIG_MOVE_MULTISTEP) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "no multi-step move is set"); }
    if ((int)h->ms_pdfs.size() >= MCIG_MAXPDF) { return set_err(MCIG_ERR_UNSUPPORTED, "at most %d sub-sampling functions", MCIG_MAXPDF); }
    int np_ = 0;
    int rc = is_user_pdf(kind) ? user_pdf_nproto(h, kind, &np_) : check_pdf(h->ndim, kind, params, nparams);
    if (rc) { return rc; }
    h->ms_pdfs.push_back(PdfDef{kind, std::vector<double>(params, params + std::max(nparams, 0))});
    return MCIG_OK;
}

extern "C" int mcig_add_sampling_function(mcig_mci *h, int kind, const double *params, int nparams)
{
    if ((int)h->pdfs.size() >= MCIG_MAXPDF) { return set_err(MCIG_ERR_UNSUPPORTED, "at most %d sampling functions", MCIG_MAXPDF); }
    int np_ = 0;
    int rc = is_user_pdf(kind) ? user_pdf_nproto(h, kind, &np_) : check_pdf(h->ndim, kind, params, nparams);
    if (rc) { return rc; }
    h->pdfs.push_back(PdfDef{kind, std::vector<double>(params, params + std::max(nparams, 0))});
    return MCIG_OK;
}

extern "C" int mcig_pop_sampling_function(mcig_mci *h)
{
    if (!h->pdfs.empty()) { h->pdfs.pop_back(); }
    return MCIG_OK;
}

extern "C" int mcig_clear_sampling_functions(mcig_mci *h)
{
    h->pdfs.clear();
    return MCIG_OK;
}

extern "C" int mcig_get_npdf(const mcig_mci *h, int *n) { *n = (int)h->pdfs.size(); return MCIG_OK; }

extern "C" int mcig_add_observable(mcig_mci *h, int kind, const double *params, int nparams, int blocksize, int nskip,
                                   int flag_equil, int estimator)
{
    if ((int)h->obs.size() >= MCIG_MAXOBS) { return set_err(MCIG_ERR_UNSUPPORTED, "at most %d observables", MCIG_MAXOBS); }
    blocksize = std::max(0, blocksize);
    nskip = std::max(1, nskip);
    if (flag_equil && estimator == MCIG_EST_NOOP) {
        return set_err(MCIG_ERR_INVALID_ARGUMENT, "[MCI::addObservable] Requested automatic observable equilibration requires estimator with error calculation.");
    }
    if (estimator < MCIG_EST_NOOP || estimator > MCIG_EST_MJBLOCKER) { return set_err(MCIG_ERR_DOMAIN, "[createEstimator] Unhandled estimator enumerator."); }
    int nv = 0;
    int rc = is_user_obs(kind) ? user_obs_nvals(h, kind, &nv) : obs_nvals(h->ndim, kind, params, nparams, &nv);
    if (rc) { return rc; }
    int maxnv = 2 * maxd_bucket(h->ndim) + 8;
    if (nobsdim(h) + nv > maxnv) { return set_err(MCIG_ERR_UNSUPPORTED, "at most %d observable values for ndim %d", maxnv, h->ndim); }
    ObsDef o;
    o.kind = kind;
    o.params.assign(params, params + std::max(nparams, 0));
    o.nv = nv;
    o.blocksize = blocksize;
    o.nskip = nskip;
    o.flag_equil = flag_equil ? 1 : 0;
    o.estimator = estimator;
    o.acc = (blocksize == 0) ? MCIG_ACC_SIMPLE : (blocksize == 1 ? MCIG_ACC_FULL : MCIG_ACC_BLOCK);
    h->obs.push_back(o);
    return MCIG_OK;
}

extern "C" int mcig_add_observable_default(mcig_mci *h, int kind, const double *params, int nparams, int blocksize, int nskip)
{
    // addObservable(obs, blocksize, nskip) -> flag_equil = blocksize > 0,
    // flag_correlated = blocksize == 1, selectEstimatorType (Factories.hpp:56-66)
    const int bs = std::max(0, blocksize);
    const int est = (bs == 1) ? MCIG_EST_CORRELATED : (bs > 0 ? MCIG_EST_UNCORRELATED : MCIG_EST_NOOP);
    return mcig_add_observable(h, kind, params, nparams, blocksize, nskip, bs > 0, est);
}

extern "C" int mcig_pop_observable(mcig_mci *h)
{
    if (!h->obs.empty()) { h->obs.pop_back(); }
    return MCIG_OK;
}

extern "C" int mcig_clear_observables(mcig_mci *h)
{
    h->obs.clear();
    return MCIG_OK;
}

extern "C" int mcig_get_nobs(const mcig_mci *h, int *n) { *n = (int)h->obs.size(); return MCIG_OK; }
extern "C" int mcig_get_nobsdim(const mcig_mci *h, int *n) { *n = nobsdim(h); return MCIG_OK; }

extern "C" int mcig_set_full_storage(mcig_mci *h, int bits)
{
    if (bits != 32 && bits != 64) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "full storage must be 32 or 64 bits"); }
    h->full32 = (bits == 32);
    return MCIG_OK;
}

extern "C" int mcig_set_irange(mcig_mci *h, const double *lb, const double *ub)
{
    for (int i = 0; i < h->ndim; ++i) {
        if (!(ub[i] > lb[i])) {
            return set_err(MCIG_ERR_INVALID_ARGUMENT, "[OrthoPeriodicDomain::checkBounds] All upper bounds must be truly greater than their corresponding lower bounds.");
        }
    }
    h->lb.assign(lb, lb + h->ndim);
    h->ub.assign(ub, ub + h->ndim);
    h->periodic = 1;
    // MCI::setIRange applies the new domain to the walkers (MCIntegrator.cpp:398-408)
    std::vector<double> x((size_t)h->nchains * h->ndim);
    int rc = mcig_get_x(h, x.data());
    if (rc) { return rc; }
    return mcig_set_x(h, x.data(), h->nchains);
}

extern "C" int mcig_reset_domain(mcig_mci *h)
{
    h->periodic = 0;
    h->lb.clear();
    h->ub.clear();
    return MCIG_OK;
}

extern "C" int mcig_set_replay(mcig_mci *h, const double *tape, int64_t stride, const int64_t *lens)
{
    cudaSetDevice(h->device);
    if (!tape) {
        h->replay = false;
        return MCIG_OK;
    }
    if (h->prec != MCIG_PREC_FP64) { return set_err(MCIG_ERR_UNSUPPORTED, "replay needs MCIG_PREC_FP64"); }
    if (stride < 1) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "tape stride must be >= 1"); }
    const size_t nc = (size_t)h->nchains;
    int rc;
    if ((rc = h->tape.alloc(nc * stride)) || (rc = h->tape_len.alloc(nc))) { return rc; }
    for (size_t c = 0; c < nc; ++c) {
        if (lens[c] < 0 || lens[c] > stride) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "tape length out of range"); }
    }
    CK(cudaMemcpyAsync(h->tape.p, tape, nc * stride * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->tape_len.p, lens, nc * sizeof(int64_t), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemsetAsync(h->tpos.p, 0, nc * sizeof(int64_t), h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->tape_stride = stride;
    h->replay = true;
    return MCIG_OK;
}

extern "C" int mcig_set_record_accepts(mcig_mci *h, int on)
{
    h->record = on != 0;
    return MCIG_OK;
}

extern "C" int mcig_get_accept_bits(const mcig_mci *h, uint8_t *bits, int64_t *nsteps)
{
    *nsteps = h->bits_steps;
    if (bits && h->bits_steps > 0) {
        cudaSetDevice(h->device);
        CK(cudaMemcpyAsync(bits, h->bits.p, (size_t)h->bits_steps * h->nchains, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
    }
    return MCIG_OK;
}

// ------------------------------------------------------------------------
// parameter upload
// ------------------------------------------------------------------------
// upper Cholesky factor U (P = U^T U) of a symmetric positive definite matrix
static bool cholesky_upper(int n, const double *P, std::vector<double> &U)
{
    std::vector<double> L((size_t)n * n, 0.);
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j <= i; ++j) {
            double s = P[i * n + j];
            for (int k = 0; k < j; ++k) { s -= L[i * n + k] * L[j * n + k]; }
            if (i == j) {
                if (!(s > 0.)) { return false; }
                L[i * n + i] = std::sqrt(s);
            } else {
                L[i * n + j] = s / L[j * n + j];
            }
        }
    }
    U.assign((size_t)n * n, 0.);
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j) { U[i * n + j] = L[j * n + i]; }
    }
    return true;
}

static int build_pdf_desc(mcig_mci *h, const PdfDef &d, std::vector<double> &P, std::vector<float> &F, PdfDesc &out)
{
    const int nd = h->ndim;
    const int fs = maxd_bucket(nd); // float blob stride, zero-padded beyond ndim
    memset(&out, 0, sizeof(out));
    out.fstride = fs;
    out.kind = d.kind;
    out.poff = (int)P.size();
    out.np = (int)d.params.size();
    P.insert(P.end(), d.params.begin(), d.params.end());
    if (is_user_pdf(d.kind)) { return user_pdf_nproto(h, d.kind, &out.nproto); }
    if (d.kind == MCIG_PDF_GAUSS_BLOCK) {
        out.b0 = (int)d.params[0];
        out.b1 = (int)d.params[1];
        out.c = 0.5 / (d.params[2] * d.params[2]);
    }
    if (d.kind == MCIG_PDF_GAUSS_MIX) { // per-component log normalisation appended after the parameters
        const int nc = (int)d.params[0];
        const double *w = d.params.data() + 1, *s = d.params.data() + 1 + nc + nc * nd;
        for (int c = 0; c < nc; ++c) {
            double l = std::log(w[c]) - 0.5 * nd * std::log(2.0 * M_PI);
            for (int i = 0; i < nd; ++i) { l -= std::log(s[c * nd + i]); }
            P.push_back(l);
        }
        out.foff = (int)F.size();
        F.push_back((float)nc);
        const double *m = d.params.data() + 1 + nc;
        for (int c = 0; c < nc; ++c) {
            F.push_back((float)P[P.size() - nc + c]);
            for (int i = 0; i < fs; ++i) { F.push_back(i < nd ? (float)m[c * nd + i] : 0.f); }
            for (int i = 0; i < fs; ++i) { F.push_back(i < nd ? (float)(1.0 / s[c * nd + i]) : 0.f); }
        }
    }
    if (d.kind == MCIG_PDF_GAUSS_PREC) {
        std::vector<double> U;
        if (!cholesky_upper(nd, d.params.data(), U)) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "GAUSS_PREC matrix is not positive definite"); }
        out.foff = (int)F.size();
        for (int i = 0; i < fs; ++i) {
            for (int j = 0; j < fs; ++j) { F.push_back((i < nd && j < nd) ? (float)U[i * nd + j] : 0.f); }
        }
    }
    return MCIG_OK;
}

// (magic, shift) with n / d == umulhi(n, magic) >> shift for every n < 2^31:
// s = floor(log2 d); a power of two uses magic 2^31 and shift s-1, any other d
// magic = floor(2^(32+s) / d) + 1 (round-up method; the rounding error of the
// reciprocal stays below 1/d for 31-bit n).  d <= 1 is never divided by.
static void magic_div(uint32_t d, uint32_t &magic, uint32_t &shift)
{
    if (d <= 1) { magic = 0; shift = 0; return; }
    uint32_t s = 0;
    while ((2ull << s) <= d) { ++s; }
    if (d == (1u << s)) { magic = 1u << 31; shift = s - 1; return; }
    magic = (uint32_t)(((1ull << (32 + s)) / d) + 1);
    shift = s;
}

// float data of the register-resident kernel at its fixed offsets (mcig_fast.cuh)
static void fill_fast_const(const mcig_mci *h, FastConst &kp)
{
    const int nd = h->ndim;
    int md = 4;
    while (md < nd) { md *= 2; }
    memset(kp.tw, 0, sizeof(kp.tw));
    for (int i = 0; i < nd && i < 32; ++i) {
        int t = 0;
        while (t + 1 < h->ntypes && i >= h->typeEnds[t]) { ++t; }
        kp.tw[t][i] = 1.f;
    }
    memset(kp.fconst, 0, sizeof(kp.fconst));
    for (const PdfDef &d : h->pdfs) {
        if (d.kind == MCIG_PDF_GAUSS_PREC) {
            std::vector<double> U;
            if (!cholesky_upper(nd, d.params.data(), U)) { continue; }
            for (int i = 0; i < nd; ++i) {
                for (int j = 0; j < nd; ++j) { kp.fconst[i * md + j] = (float)U[i * nd + j]; }
            }
        }
        if (d.kind == MCIG_PDF_GAUSS_MIX) {
            const int B = md * md, S = 1 + 2 * md;
            const int nc = (int)d.params[0];
            const double *w = d.params.data() + 1, *m = d.params.data() + 1 + nc, *sg = d.params.data() + 1 + nc + nc * nd;
            kp.fconst[B] = (float)nc;
            for (int c = 0; c < nc; ++c) {
                double l = std::log(w[c]) - 0.5 * nd * std::log(2.0 * M_PI);
                for (int i = 0; i < nd; ++i) { l -= std::log(sg[c * nd + i]); }
                kp.fconst[B + 1 + c * S] = (float)l;
                for (int i = 0; i < nd; ++i) {
                    kp.fconst[B + 1 + c * S + 1 + i] = (float)m[c * nd + i];
                    kp.fconst[B + 1 + c * S + 1 + md + i] = (float)(1.0 / sg[c * nd + i]);
                }
            }
        }
    }
}

static int fill_common(mcig_mci *h, KParams &kp)
{
    memset(&kp, 0, sizeof(kp));
    if (int rc0 = check_plugin_use(h)) { return rc0; }
    kp.ndim = h->ndim;
    kp.nchains = (int)h->nchains;
    kp.srrd = h->srrd;
    kp.veclen = h->veclen;
    kp.ntypes = h->ntypes;
    for (int i = 0; i < MCIG_MAXTYPES; ++i) { kp.typeEnds[i] = h->typeEnds[i]; }
    kp.ms_nsteps = h->ms_nsteps;
    kp.ms_srrd = h->ms_srrd;
    kp.ms_veclen = h->ms_veclen;
    std::vector<double> P;
    std::vector<float> F;
    int rc;
    if (h->movetype == MCIG_MOVE_USER) {
        kp.umove = h->umove;
        kp.umove_nproto = h->umove_nproto;
        kp.umove_poff = (int)P.size();
        kp.umove_np = (int)h->umove_params.size();
        P.insert(P.end(), h->umove_params.begin(), h->umove_params.end());
        // findMRT2Step's clamp (MCIntegrator.cpp:146-151): step size t at most 0.5 * the domain
        // size of every coordinate i with getStepSizeIndex(i) == t
        kp.step_lim_off = (int)P.size();
        for (int t = 0; t < std::max(h->ntypes, 1); ++t) {
            double lim = 0.5 * (2. * (double)3.4028234663852886e+38);
            for (int i = 0; i < h->ndim; ++i) {
                if (h->umove_stepidx[i] != t) { continue; }
                const double li = h->periodic ? 0.5 * (h->ub[i] - h->lb[i]) : 0.5 * (2. * (double)3.4028234663852886e+38);
                lim = std::min(lim, li);
            }
            P.push_back(lim);
        }
    }
    kp.npdf = (int)h->pdfs.size();
    for (int k = 0; k < kp.npdf; ++k) {
        if ((rc = build_pdf_desc(h, h->pdfs[k], P, F, kp.pdf[k]))) { return rc; }
    }
    kp.ms_npdf = (int)h->ms_pdfs.size();
    for (int k = 0; k < kp.ms_npdf; ++k) {
        if ((rc = build_pdf_desc(h, h->ms_pdfs[k], P, F, kp.ms_pdf[k]))) { return rc; }
    }
    kp.nobs = (int)h->obs.size();
    int voff = 0;
    for (int o = 0; o < kp.nobs; ++o) {
        const ObsDef &d = h->obs[o];
        ObsDesc &od = kp.obs[o];
        od.kind = d.kind;
        od.nv = d.nv;
        od.poff = (int)P.size();
        if (d.kind == MCIG_OBS_GAUSSX2) {
            P.push_back(1. / std::sqrt(M_PI * M_PI * M_PI) / 3.); // GaussXSquared::_normf (TestMCIFunctions.hpp:285)
        } else {
            P.insert(P.end(), d.params.begin(), d.params.end());
        }
        od.np = (int)d.params.size();
        od.acc = d.acc;
        od.nskip = d.nskip;
        od.bs = d.blocksize;
        od.voff = voff;
        od.full32 = h->full32;
        voff += d.nv;
    }
    kp.nobsdim = voff;
    if (P.empty()) { P.push_back(0.); }
    if ((rc = h->params.alloc(P.size()))) { return rc; }
    CK(cudaMemcpyAsync(h->params.p, P.data(), P.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    kp.params = h->params.p;
    if (!F.empty()) {
        if ((rc = h->fblob.alloc(F.size()))) { return rc; }
        CK(cudaMemcpyAsync(h->fblob.p, F.data(), F.size() * sizeof(float), cudaMemcpyHostToDevice, h->stream));
        kp.fblob = h->fblob.p;
        kp.fblob_len = (int)F.size();
    }
    kp.periodic = h->periodic;
    if (h->periodic) {
        std::vector<double> v(3 * (size_t)h->ndim);
        for (int i = 0; i < h->ndim; ++i) {
            v[i] = h->lb[i];
            v[h->ndim + i] = h->ub[i];
            v[2 * h->ndim + i] = 0.5 * (h->ub[i] - h->lb[i]);
        }
        if ((rc = h->lbub.alloc(v.size()))) { return rc; }
        CK(cudaMemcpyAsync(h->lbub.p, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        kp.lb = h->lbub.p;
        kp.ub = h->lbub.p + h->ndim;
        kp.step_max_i = h->lbub.p + 2 * h->ndim;
    }
    // UnboundDomain::getSizes = 2*FLT_MAX, so the clamp is at FLT_MAX (UnboundDomain.hpp:34)
    kp.step_max = 0.5 * (2. * (double)3.4028234663852886e+38);
    kp.x = h->x.p;
    kp.step = h->step.p;
    kp.ctr = h->ctr.p;
    kp.tpos = h->tpos.p;
    kp.nacc = h->nacc.p;
    kp.nrej = h->nrej.p;
    kp.key0 = (uint32_t)h->seed;
    kp.key1 = (uint32_t)(h->seed >> 32);
    for (int r = 0; r < 10; ++r) { // Philox round keys
        h->fc.rk[2 * r] = kp.key0 + (uint32_t)r * 0x9E3779B9u;
        h->fc.rk[2 * r + 1] = kp.key1 + (uint32_t)r * 0xBB67AE85u;
    }
    for (int o = 0; o < kp.nobs; ++o) {
        ObsDesc &od = kp.obs[o];
        magic_div((uint32_t)std::max(od.bs, 1), od.bs_magic, od.bs_shift);
        magic_div((uint32_t)od.nskip, od.sk_magic, od.sk_shift);
        od.inv_bs = 1. / (double)std::max(od.bs, 1);
    }
    fill_fast_const(h, h->fc);
    if (h->replay) {
        kp.tape = h->tape.p;
        kp.tape_stride = h->tape_stride;
        kp.tape_len = h->tape_len.p;
    }
    kp.nfind = h->nfind;
    kp.target = h->target;
    kp.status = h->status.p;
    kp.f64_decide = h->f64_decide;
    kp.dstats = h->f64_decide ? h->dstats.p : nullptr;
    return MCIG_OK;
}

// the register-resident float kernel serves all/vec moves up to 32 dimensions
// with a sampling function and observables it evaluates without exp()
static bool fast_eligible(const mcig_mci *h)
{
    if (uses_plugin(h)) { return false; }
    if (h->prec == MCIG_PREC_FP64 || h->replay || h->ndim > 32 || h->pdfs.empty()) { return false; }
    if (h->srrd != MCIG_SRRD_UNIFORM && h->srrd != MCIG_SRRD_GAUSSIAN) { return false; }
    if (h->movetype != MCIG_MOVE_ALL && h->movetype != MCIG_MOVE_VEC) { return false; }
    if (h->movetype == MCIG_MOVE_VEC && h->ndim > 16) { return false; }
    for (auto &o : h->obs) {
        if (o.kind == MCIG_OBS_GAUSSX2) { return false; }
    }
    if (maxd_bucket(h->ndim) == 32) { // 17..32 coordinates: the one-pdf kernels only
        if (h->pdfs.size() != 1) { return false; }
        const int k = h->pdfs[0].kind;
        if (k != MCIG_PDF_GAUSS && k != MCIG_PDF_GAUSS_SUM && k != MCIG_PDF_GAUSS_PREC && k != MCIG_PDF_GAUSS_MIX) { return false; }
    }
    int nprec = 0, nmix = 0; // one precision matrix and one mixture (<= 8 components) fit the parameter block
    for (auto &d : h->pdfs) {
        nprec += d.kind == MCIG_PDF_GAUSS_PREC;
        nmix += d.kind == MCIG_PDF_GAUSS_MIX;
        if (d.kind == MCIG_PDF_GAUSS_MIX && (int)d.params[0] > 8) { return false; }
    }
    return nprec <= 1 && nmix <= 1;
}

// the multi-lane mixture kernel (mcig_lanes.cuh) serves float walkers with an all-coordinate
// uniform or Gaussian move, one step type, the unbound domain, one mixture sampling function
// of at most 8 components, 17..32 coordinates and observables without exp()
static bool lanes_eligible(const mcig_mci *h)
{
    if (uses_plugin(h) || h->prec == MCIG_PREC_FP64 || h->replay || h->periodic) { return false; }
    if (h->ndim < 17 || h->ndim > 32 || h->movetype != MCIG_MOVE_ALL || h->ntypes != 1) { return false; }
    if (h->srrd != MCIG_SRRD_UNIFORM && h->srrd != MCIG_SRRD_GAUSSIAN) { return false; }
    if (h->pdfs.size() != 1 || h->pdfs[0].kind != MCIG_PDF_GAUSS_MIX || (int)h->pdfs[0].params[0] > 8) { return false; }
    for (auto &o : h->obs) {
        if (o.kind == MCIG_OBS_GAUSSX2 || o.kind == MCIG_OBS_X2BLOCK || o.kind >= MCIG_OBS_USER) { return false; }
    }
    return true;
}

// every observable of the launch is x or x.x with float Full data or a Simple/Block
// accumulator: the register-resident kernels have variants holding only those paths (1), and,
// where ndim fills the 16-coordinate kernel, every nskip is 1 and each of the four groups (Full
// x.x, Full x, Simple/Block x.x, Simple/Block x) has exactly one observable, a straight-line
// variant for that layout (2)
static int moments_only(const mcig_mci *h, const KParams &kp)
{
    int grp[4] = {0, 0, 0, 0}, nskip1 = 1;
    for (size_t o = 0; o < h->obs.size(); ++o) {
        const ObsDesc &od = kp.obs[o];
        if ((od.kind != MCIG_OBS_XND && od.kind != MCIG_OBS_X2SUM) || (od.acc == MCIG_ACC_FULL && !od.full32)) { return 0; }
        ++grp[(od.acc == MCIG_ACC_FULL ? 0 : 2) + (od.kind == MCIG_OBS_XND ? 1 : 0)];
        nskip1 &= od.nskip == 1;
    }
    const bool fixed4 = h->ndim == 16 && nskip1 && grp[0] == 1 && grp[1] == 1 && grp[2] == 1 && grp[3] == 1;
    return fixed4 ? 2 : 1;
}

// Chain counts up to which the two-lane kernel serves its configurations by default, unless
// every observable is x or x.x (then the one-lane kernel's variant for them is as fast).  One
// lane per chain fills an SM with nchains / 152 / 32 warps (3.4 at 16,384 chains, 13.5 at
// 65,536).  Measured sampling launches, 16-D precision-matrix target, 10,000 steps:
//   observables x, x.x, x_i, log p, sum x_i (general code): two lanes 18.9 against 23.9 ms at
//   16,384 chains, 25.5 against 26.8 ms at 32,768, 41.5 against 35.8 ms at 65,536;
//   x and x.x only: 18.6 / 17.9 ms at 16,384, 19.8 / 21.0 ms at 24,576, 23.4 / 21.5 ms at 32,768.
#define MCIG_PAIR_AUTO_CHAINS 32768

// the two-lane kernel (mcig_pair.cuh) serves float walkers with an all-coordinate uniform or
// Gaussian move, one step type, the unbound domain, one exp(-x.x) or precision-matrix
// sampling function, 9..16 coordinates and observables without exp() or coordinate blocks
static bool pair_eligible(const mcig_mci *h)
{
    if (uses_plugin(h) || h->prec == MCIG_PREC_FP64 || h->replay || h->periodic) { return false; }
    if (h->ndim < 9 || h->ndim > 16 || h->movetype != MCIG_MOVE_ALL || h->ntypes != 1) { return false; }
    if (h->srrd != MCIG_SRRD_UNIFORM && h->srrd != MCIG_SRRD_GAUSSIAN) { return false; }
    if (h->pdfs.size() != 1) { return false; }
    const int k = h->pdfs[0].kind;
    if (k != MCIG_PDF_GAUSS && k != MCIG_PDF_GAUSS_SUM && k != MCIG_PDF_GAUSS_PREC) { return false; }
    for (auto &o : h->obs) {
        if (o.kind == MCIG_OBS_GAUSSX2 || o.kind == MCIG_OBS_X2BLOCK || o.kind >= MCIG_OBS_USER) { return false; }
    }
    return true;
}

// the kernel family a launch of kp runs: 3 the two-lane kernel, 2 the multi-lane mixture
// kernel, 1 the register-resident one-lane kernel, 0 the general kernel (or a plugin's)
static int kernel_family(const mcig_mci *h, const KParams &kp)
{
    const bool small_n = kp.nsteps < ((int64_t)1 << 31); // 32-bit step counters in the register-resident kernels
    // two lanes per chain for burn-in and sampling (and calibration when its split tail is
    // off): mcig_set_lanes(h, 2), or automatically below MCIG_PAIR_AUTO_CHAINS chains, where
    // one lane per chain leaves the SMs with too few warps to hide latency
    const bool want_pair = h->lanes == 2 || (h->lanes == 0 && h->nchains <= MCIG_PAIR_AUTO_CHAINS && !moments_only(h, kp));
    if (kp.ndump == 0 && kp.mode != KMODE_FUSED && h->kernel_policy == 0 && want_pair && small_n &&
        pair_eligible(h) && !(kp.mode == KMODE_CALIB && h->calib_split)) {
        return 3;
    }
    // several lanes per chain: the calibration, burn-in and sampling launches of the mixture
    // configurations it serves, when asked for (mcig_set_lanes, or kernel policy 3)
    const bool want_lanes = kp.ndump == 0 && kp.mode != KMODE_FUSED &&
                            (h->kernel_policy == 3 || (h->kernel_policy == 0 && (h->lanes == 4 || h->lanes == 8)));
    if (want_lanes && small_n && lanes_eligible(h)) { return 2; }
    // file output is recorded by the general kernel
    const bool fast = kp.ndump == 0 && (h->kernel_policy == 2 || (h->kernel_policy == 0 && fast_eligible(h) && small_n));
    return fast ? 1 : 0;
}

static int launch(mcig_mci *h, const KParams &kp)
{
    const int family = kernel_family(h, kp);
    if (family == 3) {
        if (h->f64_decide) { return set_err(MCIG_ERR_UNSUPPORTED, "the FP64-certified decision runs in the multi-lane mixture kernel only (mcig_set_lanes)"); }
        const int k = h->pdfs[0].kind;
        mcig_launch_fn pf = mcig_pair_launcher(h->prec == MCIG_PREC_FP32 ? 1 : 0, k == MCIG_PDF_GAUSS_PREC ? 2 : 1,
                                               moments_only(h, kp) ? 1 : 0, h->srrd == MCIG_SRRD_GAUSSIAN);
        if (!pf) { return set_err(MCIG_ERR_UNSUPPORTED, "no two-lane kernel for this configuration"); }
        pf(kp, &h->fc, h->movetype, 0, 0, 0, h->stream);
        ++h->launches;
        CK(cudaGetLastError());
        return MCIG_OK;
    }
    if (family == 2) {
        mcig_launch_fn lf = mcig_lanes_launcher(h->prec == MCIG_PREC_FP32 ? 1 : 0, 32, h->lanes > 0 ? h->lanes : 8,
                                                h->srrd == MCIG_SRRD_GAUSSIAN);
        if (!lf) { return set_err(MCIG_ERR_UNSUPPORTED, "no multi-lane kernel for %d lanes per chain", h->lanes); }
        lf(kp, &h->fc, h->movetype, 0, 0, 0, h->stream);
        ++h->launches;
        CK(cudaGetLastError());
        return MCIG_OK;
    }
    if (h->kernel_policy == 3) { return set_err(MCIG_ERR_UNSUPPORTED, "configuration not served by the multi-lane kernel"); }
    if (h->f64_decide) { return set_err(MCIG_ERR_UNSUPPORTED, "the FP64-certified decision runs in the multi-lane mixture kernel only (mcig_set_lanes)"); }
    // 64 threads per block (MCIG_FAST_BLOCK): with ~140 registers per thread
    // seven blocks fit an SM, so 65,536 chains are resident in one wave, and
    // small batches still spread over every SM
    const int block = MCIG_FAST_BLOCK;
    const int grid = (int)((h->nchains + block - 1) / block);
    const bool small_n = kp.nsteps < ((int64_t)1 << 31);
    const bool fast = family == 1;
    mcig_launch_fn fn = nullptr;
    size_t smem = (size_t)kp.fblob_len * sizeof(float);
    if (fast) {
        if (!fast_eligible(h) || !small_n) { return set_err(MCIG_ERR_UNSUPPORTED, "configuration not served by the register-resident kernel"); }
        int pk = 0; // PK_ANY; a single sampling function of a kind with a kernel of its own
        if (h->pdfs.size() == 1) {
            const int k = h->pdfs[0].kind;
            pk = (k == MCIG_PDF_GAUSS || k == MCIG_PDF_GAUSS_SUM) ? 1 : (k == MCIG_PDF_GAUSS_PREC ? 2 : (k == MCIG_PDF_GAUSS_MIX ? 3 : 0));
        }
        const int lean = (h->ntypes == 1 && !h->periodic) ? (h->srrd == MCIG_SRRD_GAUSSIAN ? 2 : 1) : 0; // srrd: uniform or Gaussian here
        fn = mcig_fast_launcher(h->prec == MCIG_PREC_FP32 ? 1 : 0, h->movetype, maxd_bucket(h->ndim), pk, moments_only(h, kp), lean);
        smem = (size_t)kp.nobsdim * block * 8; // accumulator slots (float2 or double)
        if (kp.mode == KMODE_CALIB && h->calib_split && h->movetype == MCIG_MOVE_ALL && maxd_bucket(h->ndim) == 16 &&
            h->ntypes == 1 && !h->periodic && (pk == 1 || pk == 2)) { // PK_GAUSS, PK_PREC
            fn = mcig_calib_launcher_pk16(pk, h->srrd == MCIG_SRRD_GAUSSIAN); // same results, the tail's chains on four lanes each
            smem = 0;
        }
    } else if (uses_plugin(h)) { // the plugin's general kernel over its functors
        mcig_plugin_launch_fn pf = h->plugin ? h->plugin->launcher(h->prec, h->replay ? RNG_TAPE : RNG_PHILOX) : nullptr;
        if (!pf) { return set_err(MCIG_ERR_UNSUPPORTED, "the plugin has no kernel for this precision"); }
        const int e = pf(kp, h->movetype, grid, block, smem, h->stream);
        if (e != 0) { return set_err(MCIG_ERR_CUDA, "plugin kernel launch: %s", cudaGetErrorString((cudaError_t)e)); }
        ++h->launches;
        return MCIG_OK;
    } else {
        fn = mcig_generic_launcher(h->prec, h->replay ? RNG_TAPE : RNG_PHILOX);
    }
    if (!fn) { return set_err(MCIG_ERR_UNSUPPORTED, "no kernel for this configuration"); }
    fn(kp, &h->fc, h->movetype, grid, block, smem, h->stream);
    ++h->launches;
    CK(cudaGetLastError());
    return MCIG_OK;
}

extern "C" int mcig_set_phase_fusion(mcig_mci *h, int on)
{
    if (!h) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "handle is NULL"); }
    h->fuse_phases = on ? 1 : 0;
    return MCIG_OK;
}

extern "C" int mcig_set_calibration_split(mcig_mci *h, int on)
{
    if (!h) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "handle is NULL"); }
    h->calib_split = on ? 1 : 0;
    return MCIG_OK;
}

extern "C" int mcig_set_lanes(mcig_mci *h, int lpc)
{
    if (!h) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "handle is NULL"); }
    if (lpc < 0 || lpc > 8 || (lpc > 2 && lpc != 4 && lpc != 8)) {
        return set_err(MCIG_ERR_INVALID_ARGUMENT, "lanes per chain must be 0, 1, 2, 4 or 8");
    }
    h->lanes = lpc;
    return MCIG_OK;
}

extern "C" int mcig_set_fp64_decision(mcig_mci *h, int mode)
{
    if (!h) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "handle is NULL"); }
    if (mode < 0 || mode > 2) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "FP64 decision mode must be 0, 1 or 2"); }
    if (mode && !h->dstats.p) {
        cudaSetDevice(h->device);
        int rc = h->dstats.alloc(3);
        if (rc) { return rc; }
    }
    h->f64_decide = mode;
    return MCIG_OK;
}

extern "C" int mcig_get_decision_stats(const mcig_mci *h, int64_t *checked, int64_t *reversed, double *max_margin)
{
    if (!h) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "handle is NULL"); }
    unsigned long long v[3] = {0, 0, 0};
    if (h->dstats.p) {
        cudaSetDevice(h->device);
        CK(cudaMemcpy(v, h->dstats.p, sizeof(v), cudaMemcpyDeviceToHost));
    }
    if (checked) { *checked = (int64_t)v[0]; }
    if (reversed) { *reversed = (int64_t)v[1]; }
    if (max_margin) {
        const uint32_t b = (uint32_t)v[2];
        float f;
        memcpy(&f, &b, sizeof(f));
        *max_margin = (double)f;
    }
    return MCIG_OK;
}

extern "C" int mcig_set_kernel(mcig_mci *h, int policy)
{
    if (policy < 0 || policy > 3) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "kernel policy must be 0 (auto), 1 (general), 2 (register-resident) or 3 (multi-lane)"); }
    h->kernel_policy = policy;
    return MCIG_OK;
}

static int check_status(mcig_mci *h)
{
    int st = 0;
    CK(cudaMemcpyAsync(&st, h->status.p, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (st & 1) { return set_err(MCIG_ERR_RUNTIME, "replay tape exhausted"); }
    return MCIG_OK;
}

// ------------------------------------------------------------------------
// estimators
// ------------------------------------------------------------------------
static int run_estimator(mcig_mci *h, int est, const void *data, int is_float, int64_t n, int nv, int nchains,
                         double *d_avg, double *d_err, int ldo, int off, DBuf<double> &scratch, cudaStream_t st,
                         int64_t *launches)
{
    EstArgs a;
    a.data = data;
    a.is_float = is_float;
    a.n = n;
    a.nv = nv;
    a.nchains = nchains;
    a.avg = d_avg;
    a.err = d_err;
    a.ldo = ldo;
    a.off = off;
    a.scratch = nullptr;
    a.one_d = (nv == 1);
    const int64_t S = (int64_t)nv * nchains;
    const int block = 128;
    const int grid = (int)((S + block - 1) / block);
    if (est == MCIG_EST_CORRELATED) { est = (n > 0 && (n & (n - 1)) == 0) ? MCIG_EST_MJBLOCKER : MCIG_EST_FCBLOCKER; }
    switch (est) {
    case MCIG_EST_NOOP: est_noop_kernel<<<grid, block, 0, st>>>(a); break;
    case MCIG_EST_UNCORRELATED:
        if (n < 2) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "[UncorrelatedEstimator] n must be larger than 1"); }
        if (is_float) { est_uncorr_f32_kernel<<<grid, block, 0, st>>>(a); }
        else { est_uncorr_kernel<<<grid, block, 0, st>>>(a); }
        break;
    case MCIG_EST_FCBLOCKER:
        if (n < 50) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "FCBlockerEstimator: n must be >= 50"); }
        est_fc_kernel<<<grid, block, 0, st>>>(a);
        break;
    case MCIG_EST_MJBLOCKER: {
        if (n <= 0) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "[MJBlocker] ndata must be a natural number."); }
        if ((n & (n - 1)) != 0) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "[MJBlocker] ndata must be a power of two."); }
        int rc = scratch.alloc((size_t)n * S);
        if (rc) { return rc; }
        a.scratch = scratch.p;
        est_mj_kernel<<<grid, block, 0, st>>>(a);
        break;
    }
    default: return set_err(MCIG_ERR_DOMAIN, "[createEstimator] Unhandled estimator enumerator.");
    }
    if (launches) { ++*launches; }
    CK(cudaGetLastError());
    return MCIG_OK;
}

extern "C" int mcig_estimate(int device, int estimator, int64_t n, int ndim, const double *x, double *average, double *error)
{
    if (!x || !average || !error || ndim < 1) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "bad arguments"); }
    if (n < 1) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "n must be >= 1"); }
    CK(cudaSetDevice(device));
    cudaStream_t st;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    DBuf<double> d_x, d_out, scratch;
    int rc = d_x.alloc((size_t)n * ndim);
    if (!rc) { rc = d_out.alloc(2 * (size_t)ndim); }
    if (!rc) {
        // [n][ndim] with one chain is exactly the [n][nv][nchains] layout
        cudaMemcpyAsync(d_x.p, x, (size_t)n * ndim * sizeof(double), cudaMemcpyHostToDevice, st);
        rc = run_estimator(nullptr, estimator, d_x.p, 0, n, ndim, 1, d_out.p, d_out.p + ndim, ndim, 0, scratch, st, nullptr);
    }
    if (!rc) {
        cudaMemcpyAsync(average, d_out.p, ndim * sizeof(double), cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(error, d_out.p + ndim, ndim * sizeof(double), cudaMemcpyDeviceToHost, st);
        cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) { rc = set_err(MCIG_ERR_CUDA, "estimate: %s", cudaGetErrorString(e)); }
    }
    d_x.release();
    d_out.release();
    scratch.release();
    cudaStreamDestroy(st);
    return rc;
}

// ------------------------------------------------------------------------
// accumulators on a recorded walk
// ------------------------------------------------------------------------
__global__ void walk_accumulate_kernel(int kind, const double *params, int ndim, int nv, int acc, int bs, int nskip,
                                       int64_t nsteps, const double *xs, const uint8_t *accepted, double *data)
{
    // AccumulatorInterface::accumulate with _processFull / _processOld (AccumulatorInterface.cpp:31-114)
    // for one walk; a single thread walks the steps in order.
    if (blockIdx.x != 0 || threadIdx.x != 0) { return; }
    double vals[136];
    for (int j = 0; j < nv; ++j) { vals[j] = 0.; }
    int nchanged = ndim, skipidx = nskip - 1, bidx = 0;
    int64_t storeidx = 0;
    for (int64_t i = 0; i < nsteps; ++i) {
        const double *x = xs + i * ndim;
        bool store = false;
        if (accepted[i] || nchanged > 0) {
            nchanged = ndim;
            if (++skipidx == nskip) {
                skipidx = 0;
                // observableFunction of the kind, reference operation order
                switch (kind) {
                case MCIG_OBS_X2SUM: { double s = 0.; for (int k = 0; k < ndim; ++k) { s = s + x[k] * x[k]; } vals[0] = s; break; }
                case MCIG_OBS_XND: for (int k = 0; k < ndim; ++k) { vals[k] = x[k]; } break;
                case MCIG_OBS_X2: for (int k = 0; k < ndim; ++k) { vals[k] = x[k] * x[k]; } break;
                case MCIG_OBS_X2MEAN: { double s = x[0] * x[0]; for (int k = 1; k < ndim; ++k) { s = s + x[k] * x[k]; } vals[0] = s / ndim; break; }
                case MCIG_OBS_CONST: vals[0] = params[0]; break;
                case MCIG_OBS_XI: vals[0] = x[(int)params[0]]; break;
                case MCIG_OBS_POLYNOM: { double s = 0.; for (int k = 0; k < ndim; ++k) { s = s + x[k]; } vals[0] = s; break; }
                default: break;
                }
                nchanged = 0;
                store = true;
            }
        } else if (++skipidx == nskip) {
            skipidx = 0;
            store = true;
        }
        if (store) {
            if (acc == MCIG_ACC_FULL) {
                for (int j = 0; j < nv; ++j) { data[storeidx + j] = vals[j]; }
                storeidx += nv;
            } else if (acc == MCIG_ACC_SIMPLE) {
                for (int j = 0; j < nv; ++j) { data[j] = data[j] + vals[j]; }
            } else {
                for (int j = 0; j < nv; ++j) { data[storeidx + j] = data[storeidx + j] + vals[j]; }
                if (++bidx == bs) { bidx = 0; storeidx += nv; }
            }
        }
    }
    const int64_t naccu = 1 + (nsteps - 1) / nskip;
    if (acc == MCIG_ACC_SIMPLE) {
        const double normf = 1. / (double)naccu;
        for (int j = 0; j < nv; ++j) { data[j] = data[j] * normf; }
    } else if (acc == MCIG_ACC_BLOCK) {
        const double normf = 1. / bs;
        for (int64_t i = 0; i < (naccu / bs) * nv; ++i) { data[i] = data[i] * normf; }
    }
}

extern "C" int mcig_accumulate_walk(int device, int obs_kind, const double *params, int nparams, int ndim, int blocksize,
                                    int nskip, int64_t nsteps, const double *xs, const uint8_t *accepted, double *data,
                                    int64_t *ndata)
{
    if (ndim < 1 || ndim > 64 || !xs || !accepted || !ndata) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "bad arguments"); }
    int nv = 0;
    int rc = obs_nvals(ndim, obs_kind, params, nparams, &nv);
    if (rc) { return rc; }
    if (obs_kind == MCIG_OBS_X2BLOCK || obs_kind == MCIG_OBS_GAUSSX2 || obs_kind == MCIG_OBS_LOGPDF) {
        return set_err(MCIG_ERR_UNSUPPORTED, "observable kind not supported on a walk");
    }
    blocksize = std::max(0, blocksize);
    nskip = std::max(1, nskip);
    if (nsteps < 1) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "[AccumulatorInterface::allocate] Provided number of MC steps was < 1 ."); }
    const int acc = (blocksize == 0) ? MCIG_ACC_SIMPLE : (blocksize == 1 ? MCIG_ACC_FULL : MCIG_ACC_BLOCK);
    const int64_t naccu = 1 + (nsteps - 1) / nskip;
    int64_t nstore = 1;
    if (acc == MCIG_ACC_FULL) { nstore = naccu; }
    if (acc == MCIG_ACC_BLOCK) {
        if (naccu < blocksize) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "[BlockAccumulator::allocate] Requested number of accumulations is smaller than the requested block size."); }
        if (naccu % blocksize != 0) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "[BlockAccumulator::allocate] Requested number of accumulations is not a multiple of the requested block size."); }
        nstore = naccu / blocksize;
    }
    *ndata = nstore * nv;
    if (!data) { return MCIG_OK; }
    CK(cudaSetDevice(device));
    DBuf<double> d_xs, d_p, d_data;
    DBuf<uint8_t> d_acc;
    if ((rc = d_xs.alloc((size_t)nsteps * ndim)) || (rc = d_p.alloc(std::max(1, nparams))) ||
        (rc = d_data.alloc((size_t)nstore * nv)) || (rc = d_acc.alloc((size_t)nsteps))) {
        return rc;
    }
    CK(cudaMemcpy(d_xs.p, xs, (size_t)nsteps * ndim * sizeof(double), cudaMemcpyHostToDevice));
    if (nparams > 0) { CK(cudaMemcpy(d_p.p, params, nparams * sizeof(double), cudaMemcpyHostToDevice)); }
    CK(cudaMemcpy(d_acc.p, accepted, (size_t)nsteps, cudaMemcpyHostToDevice));
    CK(cudaMemset(d_data.p, 0, (size_t)nstore * nv * sizeof(double)));
    walk_accumulate_kernel<<<1, 32>>>(obs_kind, d_p.p, ndim, nv, acc, blocksize, nskip, nsteps, d_xs.p, d_acc.p, d_data.p);
    CK(cudaGetLastError());
    CK(cudaMemcpy(data, d_data.p, (size_t)nstore * nv * sizeof(double), cudaMemcpyDeviceToHost));
    d_xs.release(); d_p.release(); d_data.release(); d_acc.release();
    return MCIG_OK;
}

// ------------------------------------------------------------------------
// integrate
// ------------------------------------------------------------------------
static int64_t min_stat(int ndim)
{
    const double d = std::sqrt(40000. * ndim);
    return (int64_t)(d > 100. ? d : 100.); // MIN_STAT / MIN_NMC (MCIntegrator.cpp:107, :193)
}

static int alloc_obs_data(mcig_mci *h, const std::vector<ObsDef> &obs, int64_t nmc, std::vector<DBuf<char>> &bufs,
                          std::vector<int64_t> &nstore, int full32)
{
    bufs.resize(obs.size());
    nstore.assign(obs.size(), 0);
    for (size_t o = 0; o < obs.size(); ++o) {
        const ObsDef &d = obs[o];
        const int64_t naccu = 1 + (nmc - 1) / d.nskip;
        int64_t ns = 1;
        size_t elem = sizeof(double);
        if (d.acc == MCIG_ACC_FULL) {
            ns = naccu;
            if (full32) { elem = sizeof(float); }
        } else if (d.acc == MCIG_ACC_BLOCK) {
            ns = naccu / d.blocksize;
        }
        nstore[o] = ns;
        int rc = bufs[o].alloc((size_t)ns * d.nv * h->nchains * elem);
        if (rc) { return rc; }
    }
    return MCIG_OK;
}

static int validate_accumulators(const mcig_mci *h, int64_t nmc)
{
    for (auto &d : h->obs) { // BlockAccumulator::_allocate (BlockAccumulator.cpp:6-17)
        if (d.acc != MCIG_ACC_BLOCK) { continue; }
        const int64_t naccu = 1 + (nmc - 1) / d.nskip;
        if (naccu < d.blocksize) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "[BlockAccumulator::allocate] Requested number of accumulations is smaller than the requested block size."); }
        if (naccu % d.blocksize != 0) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "[BlockAccumulator::allocate] Requested number of accumulations is not a multiple of the requested block size."); }
    }
    for (auto &d : h->obs) {
        const int64_t ns = d.acc == MCIG_ACC_FULL ? 1 + (nmc - 1) / d.nskip : (d.acc == MCIG_ACC_BLOCK ? (1 + (nmc - 1) / d.nskip) / d.blocksize : 1);
        int e = d.estimator;
        if (e == MCIG_EST_CORRELATED) { e = (ns > 0 && (ns & (ns - 1)) == 0) ? MCIG_EST_MJBLOCKER : MCIG_EST_FCBLOCKER; }
        if (e == MCIG_EST_UNCORRELATED && ns < 2) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "[UncorrelatedEstimator] n must be larger than 1"); }
        if (e == MCIG_EST_FCBLOCKER && ns < 50) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "FCBlockerEstimator: n must be >= 50"); }
        if (e == MCIG_EST_MJBLOCKER && (ns & (ns - 1)) != 0) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "[MJBlocker] ndata must be a power of two."); }
    }
    return MCIG_OK;
}

// estimators of all observables -> per-chain avg/err (host vectors [nchains][nod])
static int estimate_all(mcig_mci *h, const std::vector<ObsDef> &obs, const std::vector<DBuf<char>> &bufs,
                        const std::vector<int64_t> &nstore, int full32, std::vector<double> &cavg, std::vector<double> &cerr,
                        bool to_host = true, const std::vector<char> *done = nullptr)
{
    int nod = 0;
    for (auto &o : obs) { nod += o.nv; }
    const size_t nc = (size_t)h->nchains;
    int rc;
    if ((rc = h->est_avg.alloc(nc * std::max(nod, 1))) || (rc = h->est_err.alloc(nc * std::max(nod, 1)))) { return rc; }
    int off = 0;
    for (size_t o = 0; o < obs.size(); ++o) {
        if (done && (*done)[o]) { // estimated chunk by chunk beside the sampling (sample_chunked)
            off += obs[o].nv;
            continue;
        }
        const int is_float = (obs[o].acc == MCIG_ACC_FULL && full32) ? 1 : 0;
        rc = run_estimator(h, obs[o].estimator, bufs[o].p, is_float, nstore[o], obs[o].nv, (int)nc, h->est_avg.p,
                           h->est_err.p, nod, off, h->scratch, h->stream, &h->launches);
        if (rc) { return rc; }
        off += obs[o].nv;
    }
    if (!to_host) { return MCIG_OK; }
    cavg.resize(nc * nod);
    cerr.resize(nc * nod);
    if (nod > 0) {
        CK(cudaMemcpyAsync(cavg.data(), h->est_avg.p, nc * nod * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaMemcpyAsync(cerr.data(), h->est_err.p, nc * nod * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
    return MCIG_OK;
}

// MPIMCI::integrate reduction (src/MPIMCI.cpp:85-92) of the per-chain estimates:
// average = sum(avg) / n, error = sqrt(sum(err^2)) / n, with a fixed summation order
// (COMB_T partial sums over the chains t, t + COMB_T, ..., then a pairwise tree) that
// the device kernel and the host function below share, so a batched integral and its
// own integrate give the same bits (this unit is compiled with -fmad=false and
// -ffp-contract=off).
#define COMB_T 256

static void combine_host(const double *avg, const double *err, int64_t stride, int64_t n, double &a, double &e)
{
    double pa[COMB_T], pe[COMB_T];
    for (int t = 0; t < COMB_T; ++t) {
        double sa = 0., se = 0.;
        for (int64_t c = t; c < n; c += COMB_T) {
            sa += avg[c * stride];
            se += err[c * stride] * err[c * stride];
        }
        pa[t] = sa;
        pe[t] = se;
    }
    for (int h = COMB_T / 2; h > 0; h >>= 1) {
        for (int t = 0; t < h; ++t) {
            pa[t] += pa[t + h];
            pe[t] += pe[t + h];
        }
    }
    a = pa[0] / (double)n;
    e = std::sqrt(pe[0]) / (double)n;
}

// one block of COMB_T threads per value i (stride nod between chains); scale: volume
// factor of the no-pdf path
static __global__ void __launch_bounds__(COMB_T) combine_chains_kernel(const double *__restrict__ avg,
                                                                      const double *__restrict__ err, int64_t nc,
                                                                      int nod, int scale, double vol, double *out)
{
    __shared__ double pa[COMB_T], pe[COMB_T];
    const int i = blockIdx.x, t = threadIdx.x;
    double sa = 0., se = 0.;
    for (int64_t c = t; c < nc; c += COMB_T) {
        sa += avg[c * nod + i];
        se += err[c * nod + i] * err[c * nod + i];
    }
    pa[t] = sa;
    pe[t] = se;
    __syncthreads();
    for (int h = COMB_T / 2; h > 0; h >>= 1) {
        if (t < h) {
            pa[t] += pa[t + h];
            pe[t] += pe[t + h];
        }
        __syncthreads();
    }
    if (t == 0) {
        double a = pa[0] / (double)nc, e = sqrt(pe[0]) / (double)nc;
        if (scale) {
            a *= vol;
            e *= vol;
        }
        out[i] = a;
        out[nod + i] = e;
    }
}

// combination of the estimates in est_avg/est_err into average/error (host arrays)
static int combine_on_device(mcig_mci *h, int nod, double *average, double *error, int scale, double vol)
{
    int rc;
    if ((rc = h->comb.alloc(2 * (size_t)std::max(nod, 1)))) { return rc; }
    if (!h->h_comb) { CK(cudaMallocHost(&h->h_comb, 2 * MCIG_MAXOBS * (2 * MCIG_MAXDIM + 8) * sizeof(double))); }
    combine_chains_kernel<<<nod, COMB_T, 0, h->stream>>>(h->est_avg.p, h->est_err.p, h->nchains, nod, scale, vol, h->comb.p);
    ++h->launches;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h->h_comb, h->comb.p, 2 * (size_t)nod * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    std::copy(h->h_comb, h->h_comb + nod, average);
    std::copy(h->h_comb + nod, h->h_comb + 2 * nod, error);
    return MCIG_OK;
}

// host copies of the last integrate's per-chain estimates and counts, made on demand
static int host_results(const mcig_mci *h)
{
    const size_t nc = (size_t)h->nchains;
    if (h->counts_on_device) {
        h->h_nacc.resize(nc);
        h->h_nrej.resize(nc);
        CK(cudaSetDevice(h->device));
        CK(cudaMemcpy(h->h_nacc.data(), h->nacc.p, nc * sizeof(int64_t), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(h->h_nrej.data(), h->nrej.p, nc * sizeof(int64_t), cudaMemcpyDeviceToHost));
        h->counts_on_device = false;
    }
    if (h->chains_on_device) {
        const size_t n = nc * (size_t)nobsdim(h);
        h->chain_avg.resize(n);
        h->chain_err.resize(n);
        CK(cudaSetDevice(h->device));
        if (n > 0) {
            CK(cudaMemcpy(h->chain_avg.data(), h->est_avg.p, n * sizeof(double), cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(h->chain_err.data(), h->est_err.p, n * sizeof(double), cudaMemcpyDeviceToHost));
        }
        if (h->chain_scale != 1.) {
            for (size_t k = 0; k < n; ++k) {
                h->chain_avg[k] *= h->chain_scale;
                h->chain_err[k] *= h->chain_scale;
            }
        }
        h->chains_on_device = false;
    }
    return MCIG_OK;
}

// MCI::initialDecorrelation automatic mode (MCIntegrator.cpp:171-243), chain by chain:
// a chain leaves the loop when its consecutive estimates agree within 2 sigma.
static int auto_decorrelation(mcig_mci *h, KParams kp)
{
    std::vector<ObsDef> eq;
    for (auto &o : h->obs) {
        if (o.flag_equil) {
            ObsDef e = o;
            e.blocksize = 1;
            e.nskip = 1;
            e.acc = MCIG_ACC_FULL;
            e.estimator = MCIG_EST_CORRELATED;
            eq.push_back(e);
        }
    }
    const int64_t MIN_NMC = min_stat(h->ndim);
    const size_t nc = (size_t)h->nchains;
    std::vector<DBuf<char>> bufs;
    std::vector<int64_t> nstore;
    int rc = alloc_obs_data(h, eq, MIN_NMC, bufs, nstore, 0);
    if (rc) { return rc; }
    if ((rc = h->active.alloc(nc))) { return rc; }
    std::vector<uint8_t> act(nc, 1);
    CK(cudaMemcpyAsync(h->active.p, act.data(), nc, cudaMemcpyHostToDevice, h->stream));
    const KParams orig = kp;
    kp.mode = KMODE_SAMPLE;
    kp.nsteps = MIN_NMC;
    kp.active = h->active.p;
    kp.nobs = (int)eq.size();
    int voff = 0;
    for (int k = 0, o = 0; k < (int)h->obs.size(); ++k) {
        if (!h->obs[k].flag_equil) { continue; }
        ObsDesc od = orig.obs[k]; // kind and parameters of the observable, Full accumulator
        od.acc = MCIG_ACC_FULL;
        od.nskip = 1;
        od.bs = 1;
        od.voff = voff;
        od.data = bufs[o].p;
        od.nstore = nstore[o];
        od.full32 = 0;
        kp.obs[o] = od;
        voff += eq[o].nv;
        ++o;
    }
    kp.nobsdim = voff;
    std::vector<double> oa, oe, na, ne;
    if ((rc = launch(h, kp))) { return rc; }
    if ((rc = estimate_all(h, eq, bufs, nstore, 0, oa, oe))) { return rc; }
    const int nod = voff;
    int64_t count = 0;
    while (true) {
        if ((rc = launch(h, kp))) { return rc; }
        count += MIN_NMC;
        if (count >= std::llabs(h->ndecorr)) { break; } // the reference warns here (:219-222)
        if ((rc = estimate_all(h, eq, bufs, nstore, 0, na, ne))) { return rc; }
        bool any = false;
        for (size_t c = 0; c < nc; ++c) {
            if (!act[c]) { continue; }
            bool loop = false;
            for (int i = 0; i < nod; ++i) {
                const size_t k = c * nod + i;
                if (std::fabs(oa[k] - na[k]) > 2 * std::sqrt(oe[k] * oe[k] + ne[k] * ne[k])) { loop = true; break; }
            }
            for (int i = 0; i < nod; ++i) {
                oa[c * nod + i] = na[c * nod + i];
                oe[c * nod + i] = ne[c * nod + i];
            }
            act[c] = loop ? 1 : 0;
            any = any || loop;
        }
        if (!any) { break; }
        CK(cudaMemcpyAsync(h->active.p, act.data(), nc, cudaMemcpyHostToDevice, h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
    for (auto &b : bufs) { b.release(); }
    return MCIG_OK;
}

// ------------------------------------------------------------------------
// file output (MCIntegrator.cpp:495-542): chain 0, during the main sampling
// ------------------------------------------------------------------------
extern "C" int mcig_store_observables_on_file(mcig_mci *h, const char *path, int freq)
{
    if (!path || freq < 1) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "file output needs a path and freq >= 1"); }
    h->obs_path = path;
    h->obs_freq = freq;
    return MCIG_OK;
}

extern "C" int mcig_clear_observable_file(mcig_mci *h)
{
    h->obs_path.clear();
    h->obs_freq = 0;
    return MCIG_OK;
}

extern "C" int mcig_store_walker_positions_on_file(mcig_mci *h, const char *path, int freq)
{
    if (!path || freq < 1) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "file output needs a path and freq >= 1"); }
    h->wlk_path = path;
    h->wlk_freq = freq;
    return MCIG_OK;
}

extern "C" int mcig_clear_walker_file(mcig_mci *h)
{
    h->wlk_path.clear();
    h->wlk_freq = 0;
    return MCIG_OK;
}

// observable values (reference operation order, double) at every recorded position
static __global__ void dump_obs_kernel(const KParams p, int64_t ndump, const double *dx, double *vals)
{
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= ndump) { return; }
    double v[2 * MCIG_MAXDIM + 8];
    for (int o = 0; o < p.nobs; ++o) {
        obs_eval<double>(p, p.obs[o], dx + k * p.ndim, v);
        for (int j = 0; j < p.obs[o].nv; ++j) { vals[k * p.nobsdim + p.obs[o].voff + j] = v[j]; }
    }
}

// the steps whose walker the files need: every freq-th step for the walker file, and for
// the observable file the last accumulation step of each observable at or before every
// freq-th step (an accumulator holds the values of its last accumulation, AccumulatorInterface.cpp:99-114)
static std::vector<int64_t> dump_list(const mcig_mci *h, int64_t nmc)
{
    std::vector<int64_t> v;
    for (int64_t r = 0; r < nmc; ++r) {
        if (h->wlk_freq > 0 && r % h->wlk_freq == 0) { v.push_back(r); }
        if (h->obs_freq > 0 && r % h->obs_freq == 0) {
            for (auto &o : h->obs) { v.push_back(r - r % o.nskip); }
        }
    }
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    return v;
}

static int write_dump_files(mcig_mci *h, int64_t nmc, const std::vector<int64_t> &steps)
{
    const size_t nd = steps.size();
    const int nod = nobsdim(h);
    std::vector<double> xs(nd * h->ndim), vals(nd * std::max(nod, 1));
    CK(cudaMemcpy(xs.data(), h->dump_x.p, xs.size() * sizeof(double), cudaMemcpyDeviceToHost));
    if (nod > 0) { CK(cudaMemcpy(vals.data(), h->dump_vals.p, nd * nod * sizeof(double), cudaMemcpyDeviceToHost)); }
    auto index_of = [&](int64_t r) { return (size_t)(std::lower_bound(steps.begin(), steps.end(), r) - steps.begin()); };
    if (h->wlk_freq > 0) { // MCI::storeWalkerPositions (:533-542)
        FILE *f = fopen(h->wlk_path.c_str(), "w");
        if (!f) { return set_err(MCIG_ERR_RUNTIME, "cannot open %s", h->wlk_path.c_str()); }
        for (int64_t r = 0; r < nmc; r += h->wlk_freq) {
            const double *x = xs.data() + index_of(r) * h->ndim;
            fprintf(f, "%lld", (long long)r);
            for (int j = 0; j < h->ndim; ++j) { fprintf(f, "   %g", x[j]); }
            fprintf(f, "\n");
        }
        fclose(f);
    }
    if (h->obs_freq > 0) { // MCI::storeObservables (:509-516), ObservableContainer::printObsValues (:85-93)
        FILE *f = fopen(h->obs_path.c_str(), "w");
        if (!f) { return set_err(MCIG_ERR_RUNTIME, "cannot open %s", h->obs_path.c_str()); }
        for (int64_t r = 0; r < nmc; r += h->obs_freq) {
            fprintf(f, "%lld", (long long)r);
            int off = 0;
            for (auto &o : h->obs) {
                const double *v = vals.data() + index_of(r - r % o.nskip) * nod + off;
                for (int j = 0; j < o.nv; ++j) { fprintf(f, " %g", v[j]); }
                off += o.nv;
            }
            fprintf(f, " \n");
        }
        fclose(f);
    }
    return MCIG_OK;
}

extern "C" int mcig_set_sampling_chunks(mcig_mci *h, int n)
{
    if (!h) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "handle is NULL"); }
    if (n < 1 || n > MCIG_MAX_CHUNKS) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "chunks must be in [1, %d]", MCIG_MAX_CHUNKS); }
    h->chunks = n;
    return MCIG_OK;
}

static int64_t gcd64(int64_t a, int64_t b) { return b ? gcd64(b, a % b) : a; }

// MCI::sample of the main run (MCIntegrator.cpp:290-321) as one launch, or, where the
// register-resident kernel samples and float Full samples take the Uncorrelated estimator,
// as h->chunks launches of equal length (a multiple of every block length, so no block
// spans two launches): the estimator of each finished chunk's Full rows runs on a
// low-priority stream beside the next chunk's sampling, which is bound by instruction issue
// and leaves HBM bandwidth and issue slots to it.  Results are those of one launch and of
// the one-pass estimator (same Philox counters, accumulation indices and Kahan add order).
static int sample_chunked(mcig_mci *h, const KParams &kp, int64_t nmc, std::vector<char> &est_done)
{
    KParams s = kp;
    s.mode = KMODE_SAMPLE;
    for (size_t o = 0; o < h->obs.size(); ++o) {
        s.obs[o].data = h->obsdata[o].p;
        s.obs[o].nstore = h->obs_nstore[o];
    }
    bool chunk = h->chunks > 1 && kernel_family(h, s) == 1 && h->full32;
    int64_t q = 1; // chunk lengths are multiples of q
    bool any_full = false;
    for (auto &o : h->obs) {
        if (o.acc == MCIG_ACC_SIMPLE) { chunk = false; }
        const int64_t unit = o.acc == MCIG_ACC_BLOCK ? (int64_t)o.blocksize * o.nskip : o.nskip;
        q = q / gcd64(q, unit) * unit;
        any_full |= o.acc == MCIG_ACC_FULL && o.estimator == MCIG_EST_UNCORRELATED;
    }
    const int64_t len = q * ((nmc / h->chunks + q - 1) / q);
    chunk = chunk && any_full && len < nmc && q <= nmc / 2;
    int rc;
    if (!chunk) {
        s.nsteps = nmc;
        return launch(h, s);
    }
    if (!h->est_stream) {
        int prio_low = 0, prio_high = 0;
        cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
        CK(cudaStreamCreateWithPriority(&h->est_stream, cudaStreamNonBlocking, prio_low));
        for (auto &e : h->cev) { CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming)); }
    }
    // estimator outputs and the running Kahan sums of every chunk-estimated series
    int nod = 0;
    size_t nstate = 0;
    for (auto &o : h->obs) {
        nod += o.nv;
        if (o.acc == MCIG_ACC_FULL && o.estimator == MCIG_EST_UNCORRELATED) { nstate += (size_t)o.nv * h->nchains; }
    }
    const size_t nc = (size_t)h->nchains;
    if ((rc = h->est_avg.alloc(nc * std::max(nod, 1))) || (rc = h->est_err.alloc(nc * std::max(nod, 1))) ||
        (rc = h->est_state.alloc(nstate))) {
        return rc;
    }
    int nsm = 0;
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, h->device));
    int j = 0;
    for (int64_t r0 = 0; r0 < nmc; r0 += len, ++j) {
        s.nsteps = std::min(len, nmc - r0);
        s.r0 = r0;
        s.acc_counts = r0 > 0;
        if ((rc = launch(h, s))) { return rc; }
        CK(cudaEventRecord(h->cev[j], h->stream));
        CK(cudaStreamWaitEvent(h->est_stream, h->cev[j], 0));
        size_t soff = 0;
        int off = 0;
        for (size_t o = 0; o < h->obs.size(); ++o) {
            const ObsDef &d = h->obs[o];
            if (d.acc == MCIG_ACC_FULL && d.estimator == MCIG_EST_UNCORRELATED) {
                EstArgs a;
                memset(&a, 0, sizeof(a));
                a.data = h->obsdata[o].p;
                a.is_float = 1;
                a.n = h->obs_nstore[o];
                a.nv = d.nv;
                a.nchains = (int)nc;
                a.avg = h->est_avg.p;
                a.err = h->est_err.p;
                a.ldo = nod;
                a.off = off;
                a.one_d = (d.nv == 1);
                // rows of the accumulations of steps [r0, r0 + nsteps)
                const int64_t i0 = (r0 + d.nskip - 1) / d.nskip, i1 = (r0 + s.nsteps + d.nskip - 1) / d.nskip;
                est_uncorr_f32_chunk_kernel<<<2 * nsm, 128, 0, h->est_stream>>>(a, i0, i1, h->est_state.p + soff);
                ++h->launches;
                CK(cudaGetLastError());
                est_done[o] = 1;
                soff += (size_t)d.nv * nc;
            }
            off += d.nv;
        }
    }
    CK(cudaEventRecord(h->cev[MCIG_MAX_CHUNKS], h->est_stream)); // joined before the other estimators
    return MCIG_OK;
}

extern "C" int mcig_integrate(mcig_mci *h, int64_t nmc, double *average, double *error, int do_find, int do_decorr)
{
    if (!h) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "handle is NULL"); }
    if (h->pdfs.empty() && !h->periodic) {
        return set_err(MCIG_ERR_DOMAIN, "[MCI::integrate] Integrating over an infinite domain requires a sampling function.");
    }
    if (h->replay && h->prec != MCIG_PREC_FP64) { return set_err(MCIG_ERR_UNSUPPORTED, "replay needs MCIG_PREC_FP64"); }
    int rc;
    if (nmc > 0 && (rc = validate_accumulators(h, nmc))) { return rc; }
    if (nmc > 0 && (!average || !error) && nobsdim(h) > 0) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "average/error are NULL"); }
    CK(cudaSetDevice(h->device));
    h->launches = 0;
    for (double &m : h->ms) { m = 0.; }
    CK(cudaMemsetAsync(h->status.p, 0, sizeof(int), h->stream));
    if (h->f64_decide) { CK(cudaMemsetAsync(h->dstats.p, 0, 3 * sizeof(unsigned long long), h->stream)); }
    KParams kp;
    if ((rc = fill_common(h, kp))) { return rc; }
    // device buffers first, so that allocation stays outside the timed phases
    if (nmc > 0 && (rc = alloc_obs_data(h, h->obs, nmc, h->obsdata, h->obs_nstore, h->full32))) { return rc; }
    std::vector<int64_t> dump;
    if (nmc > 0 && (h->obs_freq > 0 || h->wlk_freq > 0)) {
        dump = dump_list(h, nmc);
        if ((rc = h->dump_steps.alloc(dump.size())) || (rc = h->dump_x.alloc(dump.size() * h->ndim)) ||
            (rc = h->dump_vals.alloc(dump.size() * std::max(nobsdim(h), 1)))) {
            return rc;
        }
        CK(cudaMemcpyAsync(h->dump_steps.p, dump.data(), dump.size() * sizeof(int64_t), cudaMemcpyHostToDevice, h->stream));
    }
    CK(cudaEventRecord(h->ev[0], h->stream));
    // the three phases in one launch of the register-resident kernel, where that kernel
    // serves each of them (fixed burn-in, no file output): every chain runs
    // findMRT2Step, initialDecorrelation and sample one after the other on its own
    // MCI::findMRT2Step returns at once for a move without step sizes (MCIntegrator.cpp:94)
    const bool calib = !h->pdfs.empty() && do_find && h->nfind != 0 && nstepsizes(h) > 0;
    const bool burnin = !h->pdfs.empty() && do_decorr && h->ndecorr > 0;
    const int64_t lim = (int64_t)1 << 31;
    const bool fuse = h->fuse_phases && nmc > 0 && nmc < lim && h->ndecorr < lim && dump.empty() && !h->record &&
                      !(do_decorr && h->ndecorr < 0) && h->kernel_policy != 1 && fast_eligible(h);
    if (fuse) {
        KParams s = kp;
        s.mode = KMODE_FUSED;
        s.nsteps = nmc;
        s.fuse_calib = calib ? min_stat(h->ndim) : 0;
        s.fuse_burnin = burnin ? h->ndecorr : 0;
        for (size_t o = 0; o < h->obs.size(); ++o) {
            s.obs[o].data = h->obsdata[o].p;
            s.obs[o].nstore = h->obs_nstore[o];
        }
        CK(cudaEventRecord(h->ev[1], h->stream)); // the phases' time is reported as sampling time
        CK(cudaEventRecord(h->ev[2], h->stream));
        if ((rc = launch(h, s))) { return rc; }
    }
    // phase 1: MCI::findMRT2Step (only with a pdf; every move here has step sizes)
    if (!fuse && calib) {
        KParams c = kp;
        c.mode = KMODE_CALIB;
        c.nsteps = min_stat(h->ndim);
        if ((rc = launch(h, c))) { return rc; }
    }
    if (!fuse) { CK(cudaEventRecord(h->ev[1], h->stream)); }
    // phase 2: MCI::initialDecorrelation
    if (!fuse && !h->pdfs.empty() && do_decorr) {
        if (h->ndecorr > 0) {
            KParams d = kp;
            d.mode = KMODE_STEPS;
            d.nsteps = h->ndecorr;
            if ((rc = launch(h, d))) { return rc; }
        } else if (h->ndecorr < 0) {
            if ((rc = auto_decorrelation(h, kp))) { return rc; }
        }
    }
    if (!fuse) { CK(cudaEventRecord(h->ev[2], h->stream)); }
    std::vector<char> est_done(h->obs.size(), 0);
    if (nmc > 0 && !fuse && dump.empty() && !h->record) {
        if ((rc = sample_chunked(h, kp, nmc, est_done))) { return rc; }
    } else if (nmc > 0 && !fuse) {
        KParams s = kp;
        s.mode = KMODE_SAMPLE;
        s.nsteps = nmc;
        for (size_t o = 0; o < h->obs.size(); ++o) {
            s.obs[o].data = h->obsdata[o].p;
            s.obs[o].nstore = h->obs_nstore[o];
        }
        if (h->record) {
            if ((rc = h->bits.alloc((size_t)nmc * h->nchains))) { return rc; }
            s.bits = h->bits.p;
            h->bits_steps = nmc;
        }
        if (!dump.empty()) {
            s.dump_steps = h->dump_steps.p;
            s.ndump = (int64_t)dump.size();
            s.dump_x = h->dump_x.p;
        }
        if ((rc = launch(h, s))) { return rc; }
        if (!dump.empty() && nobsdim(h) > 0) {
            dump_obs_kernel<<<(int)((dump.size() + 127) / 128), 128, 0, h->stream>>>(s, (int64_t)dump.size(), h->dump_x.p,
                                                                                  h->dump_vals.p);
            ++h->launches;
        }
    }
    CK(cudaEventRecord(h->ev[3], h->stream));
    if (std::find(est_done.begin(), est_done.end(), 1) != est_done.end()) { // the chunk estimators' stream
        CK(cudaStreamWaitEvent(h->stream, h->cev[MCIG_MAX_CHUNKS], 0));
    }
    if (nmc > 0) {
        if ((rc = estimate_all(h, h->obs, h->obsdata, h->obs_nstore, h->full32, h->chain_avg, h->chain_err, false,
                               &est_done))) {
            return rc;
        }
    }
    CK(cudaEventRecord(h->ev[4], h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if ((rc = check_status(h))) { return rc; }
    for (int k = 0; k < 4; ++k) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, h->ev[k], h->ev[k + 1]);
        h->ms[k] = ms;
    }
    h->counts_on_device = true;
    if (!dump.empty() && (rc = write_dump_files(h, nmc, dump))) { return rc; }
    if (nmc > 0) {
        // volume scaling of the no-pdf path (MCIntegrator.cpp:70-77)
        double vol = 1.;
        if (h->pdfs.empty()) {
            for (int i = 0; i < h->ndim; ++i) { vol *= (h->ub[i] - h->lb[i]); }
        }
        h->chain_scale = h->pdfs.empty() ? vol : 1.;
        h->chains_on_device = true;
        const int nod = nobsdim(h);
        if (nod > 0 && (rc = combine_on_device(h, nod, average, error, h->pdfs.empty() ? 1 : 0, vol))) { return rc; }
    }
    return MCIG_OK;
}

extern "C" int mcig_get_chain_results(const mcig_mci *h, double *chain_avg, double *chain_err)
{
    int rc = host_results(h);
    if (rc) { return rc; }
    if (chain_avg) { std::copy(h->chain_avg.begin(), h->chain_avg.end(), chain_avg); }
    if (chain_err) { std::copy(h->chain_err.begin(), h->chain_err.end(), chain_err); }
    return MCIG_OK;
}

extern "C" int mcig_get_acceptance_rate(const mcig_mci *h, double *rate)
{
    int rc = host_results(h);
    if (rc) { return rc; }
    int64_t a = 0, r = 0;
    for (size_t c = 0; c < h->h_nacc.size(); ++c) {
        a += h->h_nacc[c];
        r += h->h_nrej[c];
    }
    *rate = (a > 0) ? (double)a / ((double)a + (double)r) : 0.;
    return MCIG_OK;
}

extern "C" int mcig_get_counts(const mcig_mci *h, int64_t *acc, int64_t *rej)
{
    int rc = host_results(h);
    if (rc) { return rc; }
    std::copy(h->h_nacc.begin(), h->h_nacc.end(), acc);
    std::copy(h->h_nrej.begin(), h->h_nrej.end(), rej);
    return MCIG_OK;
}

extern "C" int mcig_get_obs_data(const mcig_mci *h, int o, double *data, int64_t *n)
{
    if (o < 0 || o >= (int)h->obsdata.size() || o >= (int)h->obs.size()) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "no data for observable %d", o); }
    const ObsDef &d = h->obs[o];
    const int64_t ns = h->obs_nstore[o];
    const size_t nc = (size_t)h->nchains;
    *n = ns * d.nv * (int64_t)nc;
    if (!data) { return MCIG_OK; }
    cudaSetDevice(h->device);
    const bool f32 = (d.acc == MCIG_ACC_FULL && h->full32);
    const size_t cnt = (size_t)ns * d.nv * nc;
    std::vector<double> t(cnt);
    if (f32) {
        std::vector<float> tf(cnt);
        CK(cudaMemcpy(tf.data(), h->obsdata[o].p, cnt * sizeof(float), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < cnt; ++i) { t[i] = tf[i]; }
    } else {
        CK(cudaMemcpy(t.data(), h->obsdata[o].p, cnt * sizeof(double), cudaMemcpyDeviceToHost));
    }
    for (size_t c = 0; c < nc; ++c) {
        for (int64_t i = 0; i < ns; ++i) {
            for (int j = 0; j < d.nv; ++j) { data[(c * ns + i) * d.nv + j] = t[((size_t)i * d.nv + j) * nc + c]; }
        }
    }
    return MCIG_OK;
}

extern "C" int mcig_get_obs_data_chains(const mcig_mci *h, int o, int64_t c0, int64_t nc, double *data, int64_t *n)
{
    if (o < 0 || o >= (int)h->obsdata.size() || o >= (int)h->obs.size()) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "no data for observable %d", o); }
    if (c0 < 0 || nc < 0 || c0 + nc > h->nchains) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "chains [%lld, %lld) outside [0, %lld)", (long long)c0, (long long)(c0 + nc), (long long)h->nchains); }
    const ObsDef &d = h->obs[o];
    const int64_t ns = h->obs_nstore[o];
    *n = ns * d.nv * nc;
    if (!data || nc == 0) { return MCIG_OK; }
    cudaSetDevice(h->device);
    const bool f32 = (d.acc == MCIG_ACC_FULL && h->full32);
    const size_t esz = f32 ? sizeof(float) : sizeof(double);
    const size_t rows = (size_t)ns * d.nv; // each row [nchains] holds one value of every chain
    std::vector<char> t(rows * (size_t)nc * esz);
    // one strided copy: nc chains of every (sample, value) row
    CK(cudaMemcpy2D(t.data(), (size_t)nc * esz, h->obsdata[o].p + (size_t)c0 * esz, (size_t)h->nchains * esz,
                    (size_t)nc * esz, rows, cudaMemcpyDeviceToHost));
    for (int64_t c = 0; c < nc; ++c) {
        for (size_t r = 0; r < rows; ++r) {
            const size_t k = r * (size_t)nc + (size_t)c;
            data[(size_t)c * rows + r] = f32 ? (double)((const float *)t.data())[k] : ((const double *)t.data())[k];
        }
    }
    return MCIG_OK;
}

extern "C" int mcig_get_step_counters(const mcig_mci *h, uint64_t *ctr)
{
    if (!h || !ctr) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "handle or ctr is NULL"); }
    cudaSetDevice(h->device);
    CK(cudaMemcpy(ctr, h->ctr.p, (size_t)h->nchains * sizeof(uint64_t), cudaMemcpyDeviceToHost));
    return MCIG_OK;
}

extern "C" int mcig_get_last_timings(const mcig_mci *h, double *ms4, int64_t *nlaunches)
{
    for (int k = 0; k < 4; ++k) { ms4[k] = h->ms[k]; }
    if (nlaunches) { *nlaunches = h->launches; }
    return MCIG_OK;
}

__global__ void philox_block_kernel(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1, uint32_t *out)
{
    const P4 q = philox4x32_10(c0, c1, c2, c3, k0, k1);
    out[0] = q.a; out[1] = q.b; out[2] = q.c; out[3] = q.d;
}

extern "C" int mcig_philox_block(int device, const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    CK(cudaSetDevice(device));
    DBuf<uint32_t> d;
    int rc = d.alloc(4);
    if (rc) { return rc; }
    philox_block_kernel<<<1, 1>>>(ctr[0], ctr[1], ctr[2], ctr[3], key[0], key[1], d.p);
    CK(cudaGetLastError());
    CK(cudaMemcpy(out, d.p, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    d.release();
    return MCIG_OK;
}

// ------------------------------------------------------------------------
// learned proposal: independence Metropolis-Hastings with the flow (mcig_flow.cu)
// ------------------------------------------------------------------------
struct mcig_flow;
int mcig_flow_pass_device(mcig_flow *f, int dir, const float *d_in, int64_t n, float *d_out, float *d_logq, float *d_tape,
                          cudaStream_t st);
int mcig_flow_train_device(mcig_flow *f, const float *d_x, int64_t nsrc, int steps, int batch, double lr, float *last_loss,
                           cudaStream_t st);
int mcig_flow_pass_device_cm(mcig_flow *f, int dir, const float *d_in, const double *in_cm, int64_t nstride, int64_t n,
                             float *out_cm, float *d_logq, cudaStream_t st);
int mcig_flow_dim(const mcig_flow *f);
int mcig_flow_propose_device(mcig_flow *f, uint64_t cycle, uint32_t key0, uint32_t key1, int64_t nstride, int64_t n,
                             float *out_cm, float *d_logq, cudaStream_t st);
int mcig_flow_density_cmf_device(mcig_flow *f, const float *in_cmf, int64_t nstride, int64_t n, float *d_logq,
                                 cudaStream_t st);
int mcig_flow_check_status(mcig_flow *f, cudaStream_t st);
int mcig_flow_density2_device(mcig_flow *f, const double *in_cm, const float *in_cmf_b, int64_t nstride, int64_t n,
                              float *logq_a, float *logq_b, cudaStream_t st);


// walkers [ndim][nchains] (double) -> rows [nchains][ndim] (float)
__global__ void walkers_to_rows_kernel(const double *x, int ndim, int nc, float *out)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nc) { return; }
    for (int i = 0; i < ndim; ++i) { out[(size_t)c * ndim + i] = (float)x[(size_t)i * nc + c]; }
}

// Metropolis-Hastings test of the flow proposal x' for every chain:
//   log u <= [log p(x') - log p(x)] + [log q(x) - log q(x')],
// then the Full accumulators record the observables at the chain's position
// (row `krow`, every observable has nskip 1 in this mode; krow < 0 records nothing).
__global__ void flow_accept_kernel(KParams p, const float *xprop, const float *lq_prop, const float *lq_cur, uint64_t cycle,
                                   int64_t krow, int64_t *nacc_flow)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= p.nchains) { return; }
    float x[MCIG_MAXDIM], xp[MCIG_MAXDIM];
    for (int i = 0; i < p.ndim; ++i) { // both chain-minor
        x[i] = (float)p.x[(size_t)i * p.nchains + c];
        xp[i] = xprop[(size_t)i * p.nchains + c];
    }
    float dl = lq_cur[c] - lq_prop[c];
    for (int k = 0; k < p.npdf; ++k) { dl += pdf_logp_f(p, p.pdf[k], xp, p.fblob) - pdf_logp_f(p, p.pdf[k], x, p.fblob); }
    const P4 q = philox4x32_10((uint32_t)cycle, (uint32_t)(cycle >> 32), (uint32_t)c, TAG_FLOW_ACCEPT << 12,
                               p.key0 ^ 0x6A09E667u, p.key1 ^ 0xBB67AE85u);
    const bool acc = isfinite(dl) && (__log2f(accept_draw<float>(q)) <= dl * 1.44269504f);
    if (acc) {
        for (int i = 0; i < p.ndim; ++i) {
            x[i] = xp[i];
            p.x[(size_t)i * p.nchains + c] = (double)xp[i];
        }
        nacc_flow[c] += 1;
    }
    if (krow < 0) { return; }
    float vals[2 * MCIG_MAXDIM + 8];
    for (int o = 0; o < p.nobs; ++o) {
        const ObsDesc &od = p.obs[o];
        obs_eval<float>(p, od, x, vals, p.fblob);
        const size_t base = (size_t)krow * od.nv * p.nchains + c;
        for (int j = 0; j < od.nv; ++j) {
            if (od.full32) { ((float *)od.data)[base + (size_t)j * p.nchains] = vals[j]; }
            else { ((double *)od.data)[base + (size_t)j * p.nchains] = (double)vals[j]; }
        }
    }
}

extern "C" int mcig_integrate_flow(mcig_mci *h, mcig_flow *f, int64_t nmc, int period, int64_t refresh, int train_steps,
                                   int batch, double lr, double *average, double *error, int do_find, int do_decorr,
                                   double *flow_acceptance)
{
    if (!h || !f) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "handle or flow is NULL"); }
    if (mcig_flow_dim(f) != h->ndim) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "flow dimension differs from the integrator's"); }
    if (h->prec == MCIG_PREC_FP64 || h->replay) { return set_err(MCIG_ERR_UNSUPPORTED, "the learned proposal runs in the float precision modes"); }
    if (h->pdfs.empty()) { return set_err(MCIG_ERR_DOMAIN, "the learned proposal needs a sampling function"); }
    if (uses_plugin(h)) { return set_err(MCIG_ERR_UNSUPPORTED, "the learned proposal evaluates built-in sampling functions only"); }
    if (period < 1 || nmc < 1) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "period and nmc must be >= 1"); }
    for (auto &o : h->obs) {
        if (o.acc != MCIG_ACC_FULL || o.nskip != 1) {
            return set_err(MCIG_ERR_UNSUPPORTED, "with the learned proposal every observable uses a FullAccumulator with nskip 1");
        }
    }
    int rc;
    if ((rc = validate_accumulators(h, nmc))) { return rc; }
    CK(cudaSetDevice(h->device));
    h->launches = 0;
    for (double &m : h->ms) { m = 0.; }
    CK(cudaMemsetAsync(h->status.p, 0, sizeof(int), h->stream));
    KParams kp;
    if ((rc = fill_common(h, kp))) { return rc; }
    if ((rc = alloc_obs_data(h, h->obs, nmc, h->obsdata, h->obs_nstore, h->full32))) { return rc; }
    const size_t nc = (size_t)h->nchains;
    const int D = h->ndim;
    DBuf<float> xf, xprop, xprop2, lq_cur, lq_prop, lq_prop2;
    DBuf<int64_t> nflow;
    if ((rc = xf.alloc(nc * D)) || (rc = xprop.alloc(nc * D)) || (rc = xprop2.alloc(nc * D)) || (rc = lq_cur.alloc(nc)) ||
        (rc = lq_prop.alloc(nc)) || (rc = lq_prop2.alloc(nc)) || (rc = nflow.alloc(nc))) {
        return rc;
    }
    // the second stream of the sampling phase: the next cycle's generative pass (it depends on
    // the flow's weights and the cycle's z only, not on the walkers) runs there beside this
    // cycle's test and the next local steps, into the other of two proposal buffers
    struct Overlap {
        cudaStream_t st = nullptr;
        cudaEvent_t d2 = nullptr, gen[2] = {nullptr, nullptr}, done = nullptr;
        ~Overlap()
        {
            if (st) { cudaStreamSynchronize(st); cudaStreamDestroy(st); }
            for (cudaEvent_t e : {d2, gen[0], gen[1], done}) { if (e) { cudaEventDestroy(e); } }
        }
    } ov;
    CK(cudaStreamCreateWithFlags(&ov.st, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&ov.d2, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ov.gen[0], cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ov.gen[1], cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ov.done, cudaEventDisableTiming));
    float *xp[2] = {xprop.p, xprop2.p}, *lqp[2] = {lq_prop.p, lq_prop2.p};
    CK(cudaEventRecord(h->ev[0], h->stream));
    if (do_find && h->nfind != 0) {
        KParams c = kp;
        c.mode = KMODE_CALIB;
        c.nsteps = min_stat(h->ndim);
        if ((rc = launch(h, c))) { return rc; }
    }
    CK(cudaEventRecord(h->ev[1], h->stream));
    if (do_decorr && h->ndecorr > 0) {
        KParams d = kp;
        d.mode = KMODE_STEPS;
        d.nsteps = h->ndecorr;
        if ((rc = launch(h, d))) { return rc; }
    }
    const int tb = 128, tg = (int)((nc + tb - 1) / tb);
    KParams sp = kp;
    sp.mode = KMODE_SAMPLE;
    for (size_t o = 0; o < h->obs.size(); ++o) {
        sp.obs[o].data = h->obsdata[o].p;
        sp.obs[o].nstore = h->obs_nstore[o];
    }
    uint64_t cycle = 0;
    // the test with the sampling function's log density as straight-line code where the
    // register-resident kernel has it (one exp(-x.x), precision-matrix or mixture function)
    mcig_flow_accept_fn fast_accept = nullptr;
    if (h->pdfs.size() == 1) {
        const PdfDef &d = h->pdfs[0];
        const int pk = (d.kind == MCIG_PDF_GAUSS || d.kind == MCIG_PDF_GAUSS_SUM) ? 1 :
                       (d.kind == MCIG_PDF_GAUSS_PREC ? 2 : ((d.kind == MCIG_PDF_GAUSS_MIX && (int)d.params[0] <= 8) ? 3 : 0));
        if (pk && h->ndim <= 32) { fast_accept = mcig_flow_accept_launcher(maxd_bucket(h->ndim), pk); }
    }
    // one independence proposal for every chain; krow = Full row to record, -1 none
    // log q of the current walkers and of the proposals both come from the density pass, one
    // deterministic function, so the Metropolis-Hastings ratio uses the same q on both sides
    // (the generative pass's own log q of x' differs from it by the bf16 rounding of its MLP
    // inputs); the proposal's z is drawn inside the generative pass
    // (the density of the walkers and of the proposals in one launch where the pass kernel
    // takes two row sets).  prefetch: the next cycle follows without a training step in
    // between, so its generative pass is issued now on the second stream, after this cycle's
    // density pass (every earlier write of the weights and read of its buffer is then done)
    int64_t pending = -1; // cycle whose proposal the second stream is forming
    auto gen = [&](uint64_t cyc, cudaStream_t st) {
        return mcig_flow_propose_device(f, cyc, kp.key0 ^ 0x6A09E667u, kp.key1 ^ 0xBB67AE85u, (int64_t)nc, (int64_t)nc,
                                        xp[cyc & 1], lqp[cyc & 1], st);
    };
    auto flow_cycle = [&](int64_t krow, bool prefetch) -> int {
        int r;
        const int b = (int)(cycle & 1);
        if (pending == (int64_t)cycle) {
            CK(cudaStreamWaitEvent(h->stream, ov.gen[b], 0));
        } else if ((r = gen(cycle, h->stream))) {
            return r;
        }
        pending = -1;
        if ((r = mcig_flow_density2_device(f, h->x.p, xp[b], (int64_t)nc, (int64_t)nc, lq_cur.p, lqp[b], h->stream))) {
            return r;
        }
        if (prefetch) {
            CK(cudaEventRecord(ov.d2, h->stream));
            CK(cudaStreamWaitEvent(ov.st, ov.d2, 0));
            if ((r = gen(cycle + 1, ov.st))) { return r; }
            CK(cudaEventRecord(ov.gen[b ^ 1], ov.st));
            pending = (int64_t)cycle + 1;
        }
        if (fast_accept) {
            fast_accept(sp, &h->fc, xp[b], lqp[b], lq_cur.p, cycle, krow, nflow.p, h->stream);
        } else {
            flow_accept_kernel<<<tg, tb, 0, h->stream>>>(sp, xp[b], lqp[b], lq_cur.p, cycle, krow, nflow.p);
        }
        h->launches += 4;
        CK(cudaGetLastError());
        ++cycle;
        return MCIG_OK;
    };
    // adaptation: train_steps cycles of period-1 local steps, a snapshot of the chain
    // positions and one Adam step on `batch` rows drawn from it.  Each step sees new
    // positions, so the flow does not fit a fixed sample; from the first quarter on
    // the cycles also make (unrecorded) flow proposals, which carry chains between modes.
    for (int t = 0; t < train_steps; ++t) {
        if (period > 1) {
            KParams l = kp;
            l.mode = KMODE_STEPS;
            l.nsteps = period - 1;
            if ((rc = launch(h, l))) { return rc; }
        }
        walkers_to_rows_kernel<<<tg, tb, 0, h->stream>>>(h->x.p, D, (int)nc, xf.p);
        ++h->launches;
        if ((rc = mcig_flow_train_device(f, xf.p, (int64_t)nc, 1, batch, lr, nullptr, h->stream))) { return rc; }
        h->launches += 5;
        if (4 * t >= train_steps && (rc = flow_cycle(-1, false))) { return rc; }
    }
    CK(cudaMemsetAsync(nflow.p, 0, nc * sizeof(int64_t), h->stream));
    const uint64_t cycle0 = cycle;
    CK(cudaEventRecord(h->ev[2], h->stream));
    // sampling: period-1 recorded local steps, then one recorded flow proposal; with
    // refresh > 0 the flow takes one more Adam step every `refresh` steps
    int64_t step = 0, next_refresh = refresh > 0 ? refresh : INT64_MAX;
    std::vector<int64_t> hacc(nc);
    while (step < nmc) {
        const int64_t nloc = std::min<int64_t>(period - 1, nmc - step);
        if (nloc > 0) {
            KParams l = sp;
            l.nsteps = nloc;
            l.acc_offset = step;
            if ((rc = launch(h, l))) { return rc; }
            step += nloc;
        }
        if (step < nmc) {
            const bool trains_next = train_steps > 0 && batch > 0 && step + 1 >= next_refresh && step + 1 < nmc;
            if ((rc = flow_cycle(step, step + period < nmc && !trains_next))) { return rc; }
            ++step;
        }
        if (step >= next_refresh && step < nmc) {
            if (train_steps > 0 && batch > 0) {
                walkers_to_rows_kernel<<<tg, tb, 0, h->stream>>>(h->x.p, D, (int)nc, xf.p);
                if ((rc = mcig_flow_train_device(f, xf.p, (int64_t)nc, 1, batch, lr, nullptr, h->stream))) { return rc; }
                h->launches += 6;
            }
            next_refresh += refresh;
        }
    }
    CK(cudaEventRecord(ov.done, ov.st)); // the second stream has nothing left (a pending pass is never unused)
    CK(cudaStreamWaitEvent(h->stream, ov.done, 0));
    CK(cudaEventRecord(h->ev[3], h->stream));
    if ((rc = estimate_all(h, h->obs, h->obsdata, h->obs_nstore, h->full32, h->chain_avg, h->chain_err))) { return rc; }
    CK(cudaEventRecord(h->ev[4], h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if ((rc = mcig_flow_check_status(f, h->stream))) { return rc; }
    for (int k = 0; k < 4; ++k) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, h->ev[k], h->ev[k + 1]);
        h->ms[k] = ms;
    }
    CK(cudaMemcpy(hacc.data(), nflow.p, nc * sizeof(int64_t), cudaMemcpyDeviceToHost));
    if (flow_acceptance) {
        int64_t a = 0;
        for (int64_t v : hacc) { a += v; }
        *flow_acceptance = cycle > cycle0 ? (double)a / ((double)(cycle - cycle0) * (double)nc) : 0.;
    }
    h->h_nacc.resize(nc);
    h->h_nrej.resize(nc);
    CK(cudaMemcpy(h->h_nacc.data(), h->nacc.p, nc * sizeof(int64_t), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(h->h_nrej.data(), h->nrej.p, nc * sizeof(int64_t), cudaMemcpyDeviceToHost));
    h->counts_on_device = h->chains_on_device = false; // the host copies above are current
    h->chain_scale = 1.;
    const int nod = nobsdim(h);
    for (int i = 0; i < nod; ++i) { combine_host(h->chain_avg.data() + i, h->chain_err.data() + i, nod, (int64_t)nc, average[i], error[i]); }
    return MCIG_OK;
}

// ------------------------------------------------------------------------
// batched integration of many independent integrals (persistent kernel + graph)
// ------------------------------------------------------------------------
#define MCIG_NBUCKETS 4
static int bucket_of(int ndim) { return ndim <= 8 ? 0 : (ndim <= 16 ? 1 : (ndim <= 32 ? 2 : 3)); }

struct mcig_batch {
    std::vector<mcig_mci *> hs;
    std::vector<int64_t> nmc;
    int device = 0, prec = MCIG_PREC_FP32, rng = RNG_PHILOX;
    cudaStream_t st = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    DBuf<KParams> cfg;
    DBuf<BatchPhase> ph;
    DBuf<BatchSep> sep;
    DBuf<BatchTask> tasks;
    std::vector<BatchTask> htasks;
    DBuf<BatchLane> lanes;                // [ntasks][32]: the chain of each lane of each task
    std::vector<BatchLane> hlanes;
    std::vector<int> task_bucket;         // ndim bucket of each task (for the per-bucket unroll)
    std::vector<char> bs;                 // integral served by the block-separable sampler
    int ntasks = 0;
    int block = 128;                      // threads per block of the launch
    int unroll[MCIG_NBUCKETS] = {0, 0, 0, 0}; // sub-step loop unrolled 2^u times, per ndim bucket
    int walk = 0, nslot = 0, nundo = 0;   // shared memory per lane of the block-separable sampler
    DBuf<int> counter;
    DBuf<BatchSeries> series;
    int nseries = 0;
    DBuf<double> s_avg, s_err;
    double *h_avg = nullptr, *h_err = nullptr; // pinned
    std::vector<int> series_handle, series_slot; // series -> (handle, chain*nod + value)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    float last_ms = 0.f;
};

// Uncorrelated/Noop estimator of every batch series, one thread per series, with the
// estimator code of mcig_integrate (this unit is compiled with -fmad=false), so a
// batched integral's error is the one its own integrate computes
static __global__ void batch_estimate_kernel(const BatchSeries *__restrict__ series, int nseries, double *avg,
                                             double *err)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseries) { return; }
    const BatchSeries q = series[s];
    double a = 0., e = 0.;
    if (q.noop) { a = q.data[0]; }
    else { uncorr_core(q.n, [&](int64_t i) { return q.data[i * q.stride]; }, q.one_d, a, e); }
    avg[s] = a;
    err[s] = e;
}

void mcig_batch_estimate_launch(const BatchSeries *series, int nseries, double *avg, double *err, cudaStream_t st)
{
    batch_estimate_kernel<<<(nseries + 127) / 128, 128, 0, st>>>(series, nseries, avg, err);
}

// the block-separable form (sample_batch.cu): single-coordinate MultiStepMove whose
// sub-pdfs and sampling functions are isotropic Gaussian factors over coordinate ranges,
// observables x.x per factor (X2BLOCK) or in all (X2SUM) on the same ranges
static bool batch_sep(const mcig_mci *h, BatchSep &b)
{
    memset(&b, 0, sizeof(b));
    if (h->prec == MCIG_PREC_FP64 || h->replay || uses_plugin(h) || h->periodic || h->ntypes != 1) { return false; }
    if (h->movetype != MCIG_MOVE_MULTISTEP || h->ms_veclen != 1 || h->ms_nsteps < 1 || h->ms_nsteps > MCIG_BS_MAXNS) { return false; }
    if (h->ms_srrd != MCIG_SRRD_UNIFORM && h->ms_srrd != MCIG_SRRD_GAUSSIAN) { return false; }
    if (h->obs.size() > MCIG_BS_MAXOBS || nobsdim(h) > MCIG_BS_MAXV) { return false; }
    auto range_of = [&](int a, int e) -> int {
        for (int r = 0; r < b.nr; ++r) {
            if (b.ra[r] == a && b.rb[r] == e) { return r; }
        }
        if (b.nr >= MCIG_BS_MAXR) { return -1; }
        b.ra[b.nr] = a;
        b.rb[b.nr] = e;
        return b.nr++;
    };
    for (size_t o = 0; o < h->obs.size(); ++o) { // observables first: their values are consecutive ranges
        const ObsDef &d = h->obs[o];
        if (d.kind == MCIG_OBS_X2SUM) {
            b.orng[o] = b.nr;
            if (range_of(0, h->ndim) != b.orng[o]) { return false; }
        } else if (d.kind == MCIG_OBS_X2BLOCK) {
            b.orng[o] = b.nr;
            const int nb = (int)d.params[0];
            for (int k = 0; k < nb; ++k) {
                if (range_of((int)d.params[1 + k], (int)d.params[2 + k]) != b.orng[o] + k) { return false; }
            }
        } else {
            return false;
        }
    }
    for (auto &d : h->pdfs) {
        if (d.kind != MCIG_PDF_GAUSS_BLOCK) { return false; }
        const int r = range_of((int)d.params[0], (int)d.params[1]);
        if (r < 0) { return false; }
        b.pc[r] += (float)(1. / (2. * d.params[2] * d.params[2]));
    }
    for (auto &d : h->ms_pdfs) {
        if (d.kind != MCIG_PDF_GAUSS_BLOCK) { return false; }
        const int r = range_of((int)d.params[0], (int)d.params[1]);
        if (r < 0) { return false; }
        b.sc[r] += (float)(1. / (2. * d.params[2] * d.params[2]));
    }
    return true;
}

// the tasks' code variants from the per-bucket unroll, uploaded
static int batch_upload_tasks(mcig_batch *b)
{
    for (int t = 0; t < b->ntasks; ++t) {
        BatchTask &k = b->htasks[t];
        k.variant = b->bs[k.integral] ? 1 + b->unroll[b->task_bucket[t]] + (b->hs[k.integral]->ms_srrd == MCIG_SRRD_GAUSSIAN ? 3 : 0) : 0;
    }
    CK(cudaMemcpy(b->tasks.p, b->htasks.data(), b->ntasks * sizeof(BatchTask), cudaMemcpyHostToDevice));
    return MCIG_OK;
}

// the persistent grid: every block resident at once
static int batch_grid(const mcig_batch *b, int block)
{
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, b->device);
    const int per_sm = std::max(1, mcig_batch_blocks_per_sm(b->prec, b->rng, block, b->walk, b->nslot, b->nundo));
    const int need = (b->ntasks * 32 + block - 1) / block;
    return std::max(1, std::min(per_sm * nsm, need));
}

static int batch_build_graph(mcig_batch *b)
{
    if (b->gexec) { cudaGraphExecDestroy(b->gexec); b->gexec = nullptr; }
    if (b->graph) { cudaGraphDestroy(b->graph); b->graph = nullptr; }
    const int grid = batch_grid(b, b->block); // occupancy query before the capture starts
    CK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
    cudaMemsetAsync(b->counter.p, 0, sizeof(int), b->st);
    mcig_batch_launch(b->prec, b->rng, b->cfg.p, b->ph.p, b->sep.p, b->tasks.p, b->lanes.p, b->ntasks, b->counter.p, grid, b->block,
                      b->walk, b->nslot, b->nundo, b->st);
    if (b->nseries) {
        mcig_batch_estimate_launch(b->series.p, b->nseries, b->s_avg.p, b->s_err.p, b->st);
        cudaMemcpyAsync(b->h_avg, b->s_avg.p, b->nseries * sizeof(double), cudaMemcpyDeviceToHost, b->st);
        cudaMemcpyAsync(b->h_err, b->s_err.p, b->nseries * sizeof(double), cudaMemcpyDeviceToHost, b->st);
    }
    cudaError_t e = cudaStreamEndCapture(b->st, &b->graph);
    if (e != cudaSuccess) { return set_err(MCIG_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e)); }
    CK(cudaGraphInstantiate(&b->gexec, b->graph, 0));
    return MCIG_OK;
}

extern "C" int mcig_batch_destroy(mcig_batch *b)
{
    if (!b) { return MCIG_OK; }
    cudaSetDevice(b->device);
    if (b->st) { cudaStreamSynchronize(b->st); }
    if (b->gexec) { cudaGraphExecDestroy(b->gexec); }
    if (b->graph) { cudaGraphDestroy(b->graph); }
    b->cfg.release(); b->ph.release(); b->sep.release(); b->tasks.release(); b->lanes.release(); b->counter.release();
    b->series.release(); b->s_avg.release(); b->s_err.release();
    if (b->h_avg) { cudaFreeHost(b->h_avg); }
    if (b->h_err) { cudaFreeHost(b->h_err); }
    if (b->t0) { cudaEventDestroy(b->t0); }
    if (b->t1) { cudaEventDestroy(b->t1); }
    if (b->st) { cudaStreamDestroy(b->st); }
    delete b;
    return MCIG_OK;
}

extern "C" int mcig_batch_create(mcig_mci **handles, int n, const int64_t *nmc, int do_find, int do_decorr, mcig_batch **out)
{
    if (!handles || !nmc || n < 1 || !out) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "batch: bad arguments"); }
    *out = nullptr;
    const int dev = handles[0]->device;
    const int prec = handles[0]->prec;
    const bool replay = handles[0]->replay;
    for (int i = 0; i < n; ++i) {
        mcig_mci *h = handles[i];
        if (!h || h->device != dev) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "batch: every handle must exist on the same device"); }
        if (h->prec != prec || h->replay != replay) { return set_err(MCIG_ERR_UNSUPPORTED, "batch: every handle must use the same precision and draw source"); }
        if (h->pdfs.empty()) { return set_err(MCIG_ERR_UNSUPPORTED, "batch: every integral needs a sampling function"); }
        if (uses_plugin(h)) { return set_err(MCIG_ERR_UNSUPPORTED, "batch: plugin kinds are integrated one handle at a time"); }
        if (nmc[i] < 1 || nmc[i] >= ((int64_t)1 << 31)) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "batch: nmc must be in [1, 2^31)"); }
        if (do_decorr && h->ndecorr < 0) { return set_err(MCIG_ERR_UNSUPPORTED, "batch: automatic decorrelation is not batched (use N > 0)"); }
        for (auto &o : h->obs) {
            const bool ok = (o.estimator == MCIG_EST_UNCORRELATED && o.acc != MCIG_ACC_SIMPLE) ||
                            (o.estimator == MCIG_EST_NOOP);
            if (!ok) { return set_err(MCIG_ERR_UNSUPPORTED, "batch: observables use the Uncorrelated or Noop estimator"); }
            if (o.acc == MCIG_ACC_FULL && h->full32) { return set_err(MCIG_ERR_UNSUPPORTED, "batch: FullAccumulator data must be double"); }
        }
        int rc = validate_accumulators(h, nmc[i]);
        if (rc) { return rc; }
    }
    CK(cudaSetDevice(dev));
    mcig_batch *b = new mcig_batch();
    b->hs.assign(handles, handles + n);
    b->nmc.assign(nmc, nmc + n);
    b->device = dev;
    b->prec = prec;
    b->rng = replay ? RNG_TAPE : RNG_PHILOX;
    cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
    cudaEventCreate(&b->t0);
    cudaEventCreate(&b->t1);
    std::vector<KParams> cfg(n);
    std::vector<BatchPhase> ph(n);
    std::vector<BatchSep> sep(n);
    b->bs.assign(n, 0);
    // every chain with its cost and packing key (code variant: sampler, ndim bucket, sub-move
    // distribution); the chains are packed into tasks below
    struct ChainItem {
        double cost;
        int key, bucket;
        BatchLane lane;
    };
    std::vector<ChainItem> items;
    int rc = MCIG_OK;
    for (int i = 0; i < n && !rc; ++i) {
        mcig_mci *h = handles[i];
        if ((rc = fill_common(h, cfg[i]))) { break; }
        if ((rc = alloc_obs_data(h, h->obs, nmc[i], h->obsdata, h->obs_nstore, h->full32))) { break; }
        cudaMemsetAsync(h->status.p, 0, sizeof(int), h->stream);
        cudaStreamSynchronize(h->stream); // parameter uploads of the handle's stream
        KParams &k = cfg[i];
        k.mode = KMODE_SAMPLE;
        k.nsteps = nmc[i];
        for (size_t o = 0; o < h->obs.size(); ++o) {
            k.obs[o].data = h->obsdata[o].p;
            k.obs[o].nstore = h->obs_nstore[o];
        }
        ph[i].min_stat = min_stat(h->ndim);
        ph[i].do_find = (do_find && h->nfind != 0) ? 1 : 0;
        ph[i].ndecorr = do_decorr ? h->ndecorr : 0;
        ph[i].movetype = h->movetype;
        b->bs[i] = (b->prec != MCIG_PREC_FP64) && batch_sep(h, sep[i]);
        if (b->bs[i]) {
            b->walk = std::max(b->walk, h->ndim);
            b->nslot = std::max(b->nslot, nobsdim(h));
            b->nundo = std::max(b->nundo, h->ms_nsteps);
        }
        // cost of a chain: its steps times the work of a step
        const double per_step = b->bs[i] ? (double)(2 + 3 * h->ms_nsteps) :
                                (double)(h->ndim + 8) * (h->movetype == MCIG_MOVE_MULTISTEP ? 1 + h->ms_nsteps : 1);
        const double cost = (double)(nmc[i] + (ph[i].do_find ? 10 * ph[i].min_stat : 0) + ph[i].ndecorr) * per_step;
        const int key = (b->bs[i] ? 16 : 0) + 2 * bucket_of(h->ndim) + (h->ms_srrd == MCIG_SRRD_GAUSSIAN ? 1 : 0);
        for (int64_t c = 0; c < h->nchains; ++c) { items.push_back({cost, key, bucket_of(h->ndim), {i, (int)c}}); }
    }
    // tasks of 32 lanes: within a packing key, chains of similar cost side by side (cost
    // descending), so a warp's lanes finish together and integrals with few chains share a
    // warp; then one queue over the whole batch, longest first, so the tail holds the short items
    std::stable_sort(items.begin(), items.end(), [](const ChainItem &x, const ChainItem &y) {
        return x.key != y.key ? x.key < y.key : x.cost > y.cost;
    });
    std::vector<std::pair<double, std::pair<BatchTask, int>>> tl; // (cost, (task, first item))
    for (size_t a = 0; a < items.size();) {
        size_t e = a + 1;
        while (e < items.size() && e - a < 32 && items[e].key == items[a].key) { ++e; }
        BatchTask t{items[a].lane.integral, items[a].lane.chain, (int)(e - a), 0};
        tl.push_back({items[a].cost, {t, (int)a}});
        a = e;
    }
    std::stable_sort(tl.begin(), tl.end(), [](const std::pair<double, std::pair<BatchTask, int>> &x,
                                              const std::pair<double, std::pair<BatchTask, int>> &y) { return x.first > y.first; });
    b->ntasks = (int)tl.size();
    b->hlanes.assign((size_t)std::max(b->ntasks, 1) * 32, BatchLane{-1, -1});
    for (int t = 0; t < b->ntasks; ++t) {
        const auto &e = tl[t];
        b->htasks.push_back(e.second.first);
        b->task_bucket.push_back(items[e.second.second].bucket);
        for (int l = 0; l < e.second.first.count; ++l) { b->hlanes[(size_t)t * 32 + l] = items[e.second.second + l].lane; }
    }
    if (!rc) { rc = b->cfg.alloc(n); }
    if (!rc) { rc = b->ph.alloc(n); }
    if (!rc) { rc = b->sep.alloc(n); }
    if (!rc) { rc = b->tasks.alloc(std::max(b->ntasks, 1)); }
    if (!rc) { rc = b->lanes.alloc(b->hlanes.size()); }
    if (!rc) { rc = b->counter.alloc(1); }
    if (rc) { mcig_batch_destroy(b); return rc; }
    cudaMemcpy(b->cfg.p, cfg.data(), n * sizeof(KParams), cudaMemcpyHostToDevice);
    cudaMemcpy(b->ph.p, ph.data(), n * sizeof(BatchPhase), cudaMemcpyHostToDevice);
    cudaMemcpy(b->sep.p, sep.data(), n * sizeof(BatchSep), cudaMemcpyHostToDevice);
    cudaMemcpy(b->lanes.p, b->hlanes.data(), b->hlanes.size() * sizeof(BatchLane), cudaMemcpyHostToDevice);
    if ((rc = batch_upload_tasks(b))) { mcig_batch_destroy(b); return rc; }
    // estimator series: every (handle, observable, chain, value)
    std::vector<BatchSeries> ser;
    for (int i = 0; i < n; ++i) {
        mcig_mci *h = handles[i];
        int off = 0;
        const int nod = nobsdim(h);
        for (size_t o = 0; o < h->obs.size(); ++o) {
            const ObsDef &d = h->obs[o];
            for (int64_t c = 0; c < h->nchains; ++c) {
                for (int j = 0; j < d.nv; ++j) {
                    BatchSeries q;
                    q.data = (const double *)h->obsdata[o].p + (size_t)j * h->nchains + c;
                    q.n = h->obs_nstore[o];
                    q.stride = (int64_t)d.nv * h->nchains;
                    q.one_d = d.nv == 1;
                    q.noop = d.estimator == MCIG_EST_NOOP;
                    ser.push_back(q);
                    b->series_handle.push_back(i);
                    b->series_slot.push_back((int)(c * nod + off + j));
                }
            }
            off += d.nv;
        }
    }
    b->nseries = (int)ser.size();
    if (b->nseries) {
        if ((rc = b->series.alloc(ser.size())) || (rc = b->s_avg.alloc(ser.size())) || (rc = b->s_err.alloc(ser.size()))) {
            mcig_batch_destroy(b);
            return rc;
        }
        cudaMemcpy(b->series.p, ser.data(), ser.size() * sizeof(BatchSeries), cudaMemcpyHostToDevice);
        cudaMallocHost(&b->h_avg, ser.size() * sizeof(double));
        cudaMallocHost(&b->h_err, ser.size() * sizeof(double));
    }
    if ((rc = batch_build_graph(b))) { mcig_batch_destroy(b); return rc; }
    *out = b;
    return MCIG_OK;
}

// one run: the graph (persistent kernel + estimators + read-back), then the MPIMCI
// combination per integral; avg/err hold the integrals' results in order
extern "C" int mcig_batch_run(mcig_batch *b, double *avg, double *err)
{
    CK(cudaSetDevice(b->device));
    CK(cudaEventRecord(b->t0, b->st));
    CK(cudaGraphLaunch(b->gexec, b->st));
    CK(cudaEventRecord(b->t1, b->st));
    CK(cudaStreamSynchronize(b->st));
    cudaEventElapsedTime(&b->last_ms, b->t0, b->t1);
    if (b->rng == RNG_TAPE) { // replay tapes that ran out
        for (auto *h : b->hs) {
            int s1 = 0;
            CK(cudaMemcpy(&s1, h->status.p, sizeof(int), cudaMemcpyDeviceToHost));
            if (s1 & 1) { return set_err(MCIG_ERR_RUNTIME, "replay tape exhausted"); }
        }
    }
    // per-chain results into the handles, then combination
    for (auto *h : b->hs) {
        const int nod = nobsdim(h);
        h->chain_avg.assign((size_t)h->nchains * nod, 0.);
        h->chain_err.assign((size_t)h->nchains * nod, 0.);
    }
    for (int s = 0; s < b->nseries; ++s) {
        mcig_mci *h = b->hs[b->series_handle[s]];
        h->chain_avg[b->series_slot[s]] = b->h_avg[s];
        h->chain_err[b->series_slot[s]] = b->h_err[s];
    }
    size_t off = 0;
    for (auto *h : b->hs) {
        const int nod = nobsdim(h);
        const size_t nc = (size_t)h->nchains;
        for (int i = 0; i < nod; ++i) {
            double a, e;
            combine_host(h->chain_avg.data() + i, h->chain_err.data() + i, nod, (int64_t)nc, a, e);
            if (avg) { avg[off + i] = a; }
            if (err) { err[off + i] = e; }
        }
        off += nod;
        h->counts_on_device = true;   // copied when asked for (host_results)
        h->chains_on_device = false;  // the chain estimates were set above
        h->chain_scale = 1.;
    }
    return MCIG_OK;
}

extern "C" int mcig_batch_last_ms(const mcig_batch *b, double *ms)
{
    *ms = b->last_ms;
    return MCIG_OK;
}

extern "C" int mcig_batch_get_tuning(const mcig_batch *b, int *block, int *unroll)
{
    if (block) { *block = b->block; }
    if (unroll) {
        for (int k = 0; k < MCIG_NBUCKETS; ++k) { unroll[k] = 1 << b->unroll[k]; }
    }
    return MCIG_OK;
}

extern "C" int mcig_batch_set_tuning(mcig_batch *b, int block, const int *unroll)
{
    if (block < 32 || block > 256 || block % 32) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "batch: the block size is a multiple of 32 in [32, 256]"); }
    int u[MCIG_NBUCKETS];
    for (int k = 0; k < MCIG_NBUCKETS; ++k) {
        const int v = unroll ? unroll[k] : (1 << b->unroll[k]);
        if (v != 1 && v != 2 && v != 4) { return set_err(MCIG_ERR_INVALID_ARGUMENT, "batch: unroll factors are 1, 2 or 4"); }
        u[k] = v == 1 ? 0 : (v == 2 ? 1 : 2);
    }
    CK(cudaSetDevice(b->device));
    CK(cudaStreamSynchronize(b->st));
    b->block = block;
    for (int k = 0; k < MCIG_NBUCKETS; ++k) { b->unroll[k] = u[k]; }
    int rc = batch_upload_tasks(b);
    return rc ? rc : batch_build_graph(b);
}

// time one run of the persistent launch alone at the current tuning (ms)
static int batch_time(mcig_batch *b, float *ms)
{
    const int grid = batch_grid(b, b->block);
    CK(cudaMemsetAsync(b->counter.p, 0, sizeof(int), b->st));
    CK(cudaEventRecord(b->t0, b->st));
    mcig_batch_launch(b->prec, b->rng, b->cfg.p, b->ph.p, b->sep.p, b->tasks.p, b->lanes.p, b->ntasks, b->counter.p, grid, b->block,
                      b->walk, b->nslot, b->nundo, b->st);
    CK(cudaEventRecord(b->t1, b->st));
    CK(cudaStreamSynchronize(b->st));
    CK(cudaGetLastError());
    cudaEventElapsedTime(ms, b->t0, b->t1);
    return MCIG_OK;
}

// Autotuner: the threads per block of the launch (64, 128, 256), then, per ndim bucket with
// block-separable integrals, the unroll of the sub-step loop (1, 2, 4), each by timing the
// persistent launch alone; the choice is cached in a text file keyed by the batch's shape
// (tasks per bucket), so later batches of the same shape skip the timing.  Tuning launches
// advance the chains like any sampling run.
extern "C" int mcig_batch_autotune(mcig_batch *b, const char *cache_path)
{
    CK(cudaSetDevice(b->device));
    int per[MCIG_NBUCKETS] = {0, 0, 0, 0}, bsper[MCIG_NBUCKETS] = {0, 0, 0, 0};
    for (int t = 0; t < b->ntasks; ++t) {
        ++per[b->task_bucket[t]];
        bsper[b->task_bucket[t]] += b->bs[b->htasks[t].integral] ? 1 : 0;
    }
    std::string key = "prec" + std::to_string(b->prec);
    for (int k = 0; k < MCIG_NBUCKETS; ++k) {
        int lg = 0;
        while ((1 << lg) < per[k]) { ++lg; }
        key += "_b" + std::to_string(k) + "t2^" + std::to_string(lg) + (bsper[k] ? "s" : "g");
    }
    std::map<std::string, std::vector<int>> cache;
    if (cache_path) {
        std::ifstream in(cache_path);
        std::string k;
        int v[1 + MCIG_NBUCKETS];
        while (in >> k >> v[0] >> v[1] >> v[2] >> v[3] >> v[4]) { cache[k] = std::vector<int>(v, v + 1 + MCIG_NBUCKETS); }
    }
    int rc;
    if (cache.count(key)) {
        const std::vector<int> &v = cache[key];
        b->block = v[0];
        for (int k = 0; k < MCIG_NBUCKETS; ++k) { b->unroll[k] = v[1 + k]; }
        if ((rc = batch_upload_tasks(b))) { return rc; }
        return batch_build_graph(b);
    }
    float best = 1e30f, ms = 0.f;
    int bestb = b->block;
    for (int bsz : {64, 128, 256}) {
        b->block = bsz;
        if ((rc = batch_time(b, &ms))) { return rc; }
        if (ms < best) { best = ms; bestb = bsz; }
    }
    b->block = bestb;
    for (int k = 0; k < MCIG_NBUCKETS; ++k) {
        if (!bsper[k]) { continue; }
        int bestu = b->unroll[k];
        best = 1e30f;
        for (int u = 0; u < 3; ++u) {
            b->unroll[k] = u;
            if ((rc = batch_upload_tasks(b)) || (rc = batch_time(b, &ms))) { return rc; }
            if (ms < best) { best = ms; bestu = u; }
        }
        b->unroll[k] = bestu;
    }
    if ((rc = batch_upload_tasks(b))) { return rc; }
    if (cache_path) {
        std::vector<int> v{b->block};
        for (int k = 0; k < MCIG_NBUCKETS; ++k) { v.push_back(b->unroll[k]); }
        cache[key] = v;
        std::ofstream o(cache_path);
        for (auto &e : cache) {
            o << e.first;
            for (int x : e.second) { o << " " << x; }
            o << "\n";
        }
    }
    return batch_build_graph(b);
}
