// ref_recorder.cpp -- drives the reference library (compiled from its sources
// by oracle/ref_build.sh) through its public API and prints golden vectors as
// JSON.  Test infrastructure only; the output is committed as
// tests/golden/reference_golden.json by tests/golden/make_golden.py.
//
// Accept/reject bits of a main sampling run are read through the reference's
// own callback (MCI::setCallback, include/mci/MCIntegrator.hpp:189): the
// callback runs once in initializeSampling and once after every step
// (src/MCIntegrator.cpp:267,347), so step k's decision is the change of the
// accepted-step count, recovered exactly from getAcceptanceRate()*k.
#include "mci/MCIntegrator.hpp"
#include "mci/MultiStepMove.hpp"
#include "mci/OrthoPeriodicDomain.hpp"
#include "mci/Estimators.hpp"
#include "mci/SimpleAccumulator.hpp"
#include "mci/BlockAccumulator.hpp"
#include "mci/FullAccumulator.hpp"

#include "common/TestMCIFunctions.hpp"

extern "C" {
#include "../oracle/mci_oracle.h"
}

#include <cstdio>
#include <string>
#include <vector>
#include <unistd.h>

using namespace mci;

static void put_array(const char *name, const double *v, int64_t n, bool last = false)
{
    std::printf("\"%s\": [", name);
    for (int64_t i = 0; i < n; ++i) { std::printf("%s%.17g", i ? ", " : "", v[i]); }
    std::printf("]%s\n", last ? "" : ",");
}

static std::string bits_hex(const std::vector<int> &b)
{
    static const char *hx = "0123456789abcdef";
    std::string s;
    for (size_t i = 0; i < b.size(); i += 4) {
        int v = 0;
        for (size_t j = 0; j < 4; ++j) { v |= (i + j < b.size() && b[i + j]) ? (1 << j) : 0; }
        s.push_back(hx[v]);
    }
    return s;
}

// deterministic test series: AR(1) x_i = phi x_{i-1} + (u_i - 1/2), u from splitmix64
static uint64_t splitmix(uint64_t &s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static std::vector<double> ar1_series(uint64_t seed, int64_t n, int nd, double phi)
{
    std::vector<double> x(n * nd);
    uint64_t s = seed;
    for (int j = 0; j < nd; ++j) { x[j] = 0.; }
    for (int64_t i = 0; i < n; ++i) {
        for (int j = 0; j < nd; ++j) {
            const double u = (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
            const double prev = (i > 0) ? x[(i - 1) * nd + j] : 0.;
            x[i * nd + j] = phi * prev + (u - 0.5);
        }
    }
    return x;
}

struct RunSpec {
    const char *name;
    int ndim;
    uint64_t seed;
    int move;      // 0 all uniform, 1 all gaussian, 2 vec uniform veclen, 3 multistep, 4 typed all uniform, 5 vec gaussian,
                   // 10 + k: SRRDType k with veclen (0: all coordinates)
    int veclen;
    int pdf;       // 0 Gauss(nd), 1 ThreeDimGaussianPDF, 2 ExpNDPDF(nd), 3 none
    int obsset;    // 0 X2Sum+XND, 1 XSquared, 2 X2Sum+X2, 3 GaussXSquared
    int blocksize, nskip;
    int estim;     // EstimatorType or -1 for the flag_correlated default
    int nfind;
    int64_t ndecorr;
    int64_t nmc;
    int periodic;
    double target;
    int nbits;     // accept bits to store
};

static void run_case(const RunSpec &r, bool last)
{
    MCI mci(r.ndim);
    mci.setSeed(r.seed);
    if (r.periodic) { mci.setIRange(-2.5, 2.5); }
    switch (r.pdf) {
    case 0: mci.addSamplingFunction(Gauss(r.ndim)); break;
    case 1: mci.addSamplingFunction(ThreeDimGaussianPDF()); break;
    case 2: mci.addSamplingFunction(ExpNDPDF(r.ndim)); break;
    default: break;
    }
    int typeEnds[2] = {1, r.ndim};
    switch (r.move) {
    case 1: mci.setTrialMove(SRRDType::Gaussian); break;
    case 2: mci.setTrialMove(SRRDType::Uniform, r.veclen); break;
    case 3: {
        MultiStepMove msm(r.ndim);
        msm.setTrialMove(UniformVecMove(r.ndim, 1, 0.1));
        msm.addSamplingFunction(ExpNDPDF(r.ndim));
        mci.setTrialMove(msm);
        break;
    }
    case 4: mci.setTrialMove(SRRDType::Uniform, 0, 2, typeEnds); break;
    case 5: mci.setTrialMove(SRRDType::Gaussian, r.veclen); break;
    default:
        if (r.move >= 10) { mci.setTrialMove(static_cast<SRRDType>(r.move - 10), r.veclen); } // SRRDType move - 10
        break;
    }
    mci.setTargetAcceptanceRate(r.target);
    mci.setNfindMRT2Iterations(r.nfind);
    mci.setNdecorrelationSteps(r.ndecorr);
    auto addobs = [&](const ObservableFunctionInterface &o) {
        if (r.estim < 0) { mci.addObservable(o, r.blocksize, r.nskip); }
        else { mci.addObservable(o, r.blocksize, r.nskip, false, static_cast<EstimatorType>(r.estim)); }
    };
    switch (r.obsset) {
    case 0: addobs(X2Sum(r.ndim)); addobs(XND(r.ndim)); break;
    case 1: addobs(XSquared()); break;
    case 2: addobs(X2Sum(r.ndim)); addobs(X2(r.ndim)); break;
    case 3: addobs(GaussXSquared()); break;
    default: break;
    }
    const int nod = mci.getNObsDim();
    std::vector<double> avg(nod), err(nod);
    // calibration + burn-in first (Nmc = 0 runs them only, src/MCIntegrator.cpp:49-56)
    mci.integrate(0, avg.data(), err.data(), true, true);
    const double acc_burn = mci.getAcceptanceRate();
    std::vector<double> step(mci.getTrialMove().getNStepSizes());
    for (size_t i = 0; i < step.size(); ++i) { step[i] = mci.getMRT2Step(i); }
    std::vector<double> xstart(mci.getX(), mci.getX() + r.ndim);
    // main sampling with the callback recording accept/reject
    std::vector<int> bits;
    int64_t ncall = 0, prev = 0;
    mci.setCallback([&](const MCI &m) {
        if (ncall > 0) {
            const int64_t a = static_cast<int64_t>(m.getAcceptanceRate() * ncall + 0.5);
            if ((int64_t)bits.size() < r.nbits) { bits.push_back(a > prev ? 1 : 0); }
            prev = a;
        }
        ++ncall;
    });
    mci.integrate(r.nmc, avg.data(), err.data(), false, false);
    mci.clearCallback();
    std::printf("\"%s\": {\n", r.name);
    put_array("avg", avg.data(), nod);
    put_array("err", err.data(), nod);
    put_array("step", step.data(), step.size());
    put_array("xstart", xstart.data(), r.ndim);
    put_array("xend", mci.getX(), r.ndim);
    std::printf("\"acc_burn\": %.17g,\n", acc_burn);
    std::printf("\"acc_main\": %.17g,\n", mci.getAcceptanceRate());
    std::printf("\"nbits\": %d,\n", (int)bits.size());
    std::printf("\"bits\": \"%s\"\n", bits_hex(bits).c_str());
    std::printf("}%s\n", last ? "" : ",");
}

static std::string json_escape_file(const std::string &path)
{
    std::FILE *f = std::fopen(path.c_str(), "rb");
    std::string out;
    if (!f) { return out; }
    int ch;
    while ((ch = std::fgetc(f)) != EOF) {
        if (ch == '\n') { out += "\\n"; }
        else if (ch == '"' || ch == '\\') { out.push_back('\\'); out.push_back((char)ch); }
        else { out.push_back((char)ch); }
    }
    std::fclose(f);
    std::remove(path.c_str());
    return out;
}

// the reference's own observable and walker files of a main sampling run
// (MCI::storeObservablesOnFile / storeWalkerPositionsOnFile, src/MCIntegrator.cpp:495-542):
// Gauss(3), uniform all-move, calibration and 200 burn-in steps in a first integrate call,
// then 1,000 recorded steps with x.x (Simple, nskip 1) and x_i (Simple, nskip 3)
static void run_file_case()
{
    MCI mci(3);
    mci.setSeed(4321);
    mci.addSamplingFunction(Gauss(3));
    mci.setNfindMRT2Iterations(-50);
    mci.setNdecorrelationSteps(200);
    mci.addObservable(X2Sum(3), 0, 1, false, EstimatorType::Noop);
    mci.addObservable(XND(3), 0, 3, false, EstimatorType::Noop);
    double avg[4], err[4];
    mci.integrate(0, avg, err, true, true);
    const std::string po = "/tmp/mcig_ref_obs_" + std::to_string((long long)getpid()) + ".txt";
    const std::string pw = "/tmp/mcig_ref_wlk_" + std::to_string((long long)getpid()) + ".txt";
    mci.storeObservablesOnFile(po, 100);
    mci.storeWalkerPositionsOnFile(pw, 50);
    mci.integrate(1000, avg, err, false, false);
    std::printf("\"file_case\": {\"seed\": 4321, \"ndecorr\": 200, \"nmc\": 1000, \"obs_freq\": 100, \"wlk_freq\": 50},\n");
    std::printf("\"file_obs\": \"%s\",\n", json_escape_file(po).c_str());
    std::printf("\"file_wlk\": \"%s\",\n", json_escape_file(pw).c_str());
}

int main()
{
    std::printf("{\n");
    // engine known answers
    {
        std::mt19937_64 g(1234);
        std::vector<double> w(8);
        std::printf("\"mt64_seed1234\": [");
        for (int i = 0; i < 8; ++i) { std::printf("%s\"%llu\"", i ? ", " : "", (unsigned long long)g()); }
        std::printf("],\n");
        std::mt19937_64 g2(1234);
        std::uniform_real_distribution<double> u(0., 1.);
        for (int i = 0; i < 8; ++i) { w[i] = u(g2); }
        put_array("canonical_seed1234", w.data(), 8);
        std::mt19937_64 g3(1234);
        std::normal_distribution<double> nd;
        std::vector<double> nv(9);
        for (int i = 0; i < 9; ++i) { nv[i] = nd(g3); }
        put_array("normal_seed1234", nv.data(), 9);
        std::mt19937_64 g4(1234);
        std::uniform_int_distribution<int> ui(0, 2);
        std::vector<double> iv(16);
        for (int i = 0; i < 16; ++i) { iv[i] = ui(g4); }
        put_array("uniform_int3_seed1234", iv.data(), 16);
    }
    // the other move distributions (createSymRRD, TrialMoveInterface.hpp:113-200): 64 draws of a
    // fresh object each from mt19937_64(1234)
    {
        std::vector<double> v(64);
        auto rec = [&](const char *name, auto dist) {
            std::mt19937_64 g(1234);
            for (int i = 0; i < 64; ++i) { v[i] = dist(g); }
            put_array(name, v.data(), 64);
        };
        rec("srrd2_seed1234", createSymRRD<std::student_t_distribution<double>>());
        rec("srrd3_seed1234", createSymRRD<std::cauchy_distribution<double>>());
        rec("srrd4_seed1234", createSymRRD<SymmetrizedPRRD<std::exponential_distribution<double>>>());
        rec("srrd5_seed1234", createSymRRD<SymmetrizedPRRD<std::gamma_distribution<double>>>());
        rec("srrd6_seed1234", createSymRRD<SymmetrizedPRRD<std::weibull_distribution<double>>>());
        rec("srrd7_seed1234", createSymRRD<SymmetrizedPRRD<std::lognormal_distribution<double>>>());
        rec("srrd8_seed1234", createSymRRD<SymmetrizedPRRD<std::chi_squared_distribution<double>>>());
        rec("srrd9_seed1234", createSymRRD<SymmetrizedPRRD<std::fisher_f_distribution<double>>>());
    }
    // estimators on a fixed correlated series (test/ut1/main.cpp:251-314 pattern)
    {
        const int64_t n = 32768;
        const int nd = 2;
        std::vector<double> x = ar1_series(1337, n, nd, 0.9);
        double a[2], e[2];
        std::printf("\"series\": {\"seed\": 1337, \"n\": %lld, \"ndim\": %d, \"phi\": 0.9},\n", (long long)n, nd);
        UncorrelatedEstimator(n, nd, x.data(), a, e);
        put_array("est_uncorr_avg", a, nd); put_array("est_uncorr_err", e, nd);
        MultiDimBlockEstimator(n, nd, x.data(), 2048, a, e);
        put_array("est_block2048_avg", a, nd); put_array("est_block2048_err", e, nd);
        FCBlockerEstimator(n, nd, x.data(), a, e);
        put_array("est_fc_avg", a, nd); put_array("est_fc_err", e, nd);
        MJBlockerEstimator(n, nd, x.data(), a, e);
        put_array("est_mj_avg", a, nd); put_array("est_mj_err", e, nd);
        // 1-D versions on column 0
        std::vector<double> x1(n);
        for (int64_t i = 0; i < n; ++i) { x1[i] = x[i * nd]; }
        OneDimFCBlockerEstimator(n, x1.data(), a[0], e[0]);
        put_array("est_fc1d", a, 1); put_array("est_fc1d_err", e, 1);
        MJBlockerEstimator(n, 1, x1.data(), a, e);
        put_array("est_mj1d", a, 1); put_array("est_mj1d_err", e, 1);
        // non power of two -> Correlated uses FCBlocker
        CorrelatedEstimator(10000, nd, x.data(), a, e);
        put_array("est_corr10000_avg", a, nd); put_array("est_corr10000_err", e, nd);
        // 17-D, 4096 samples (wider MJBlocker)
        std::vector<double> y = ar1_series(7, 4096, 17, 0.5);
        double a17[17], e17[17];
        MJBlockerEstimator(4096, 17, y.data(), a17, e17);
        put_array("est_mj17_avg", a17, 17); put_array("est_mj17_err", e17, 17);
        FCBlockerEstimator(4096, 17, y.data(), a17, e17);
        put_array("est_fc17_avg", a17, 17); put_array("est_fc17_err", e17, 17);
    }
    // accumulators on a recorded walk (test/ut1/main.cpp:116-204 pattern)
    {
        const int64_t n = 4096;
        const int nd = 2;
        std::vector<double> x = ar1_series(99, n, nd, 0.8);
        std::vector<bool> accv(n);
        uint64_t s = 4242;
        for (int64_t i = 0; i < n; ++i) {
            accv[i] = (i == 0) || (splitmix(s) % 3 != 0);
            if (!accv[i]) { for (int j = 0; j < nd; ++j) { x[i * nd + j] = x[(i - 1) * nd + j]; } }
        }
        std::printf("\"walk\": {\"seed\": 99, \"accept_seed\": 4242, \"n\": %lld, \"ndim\": %d, \"phi\": 0.8},\n", (long long)n, nd);
        XND obs(nd);
        struct { const char *name; int bs, skip; } cfg[] = {{"acc_simple_1", 0, 1}, {"acc_simple_2", 0, 2},
                                                           {"acc_block16_1", 16, 1}, {"acc_block8_2", 8, 2},
                                                           {"acc_full_1", 1, 1}, {"acc_full_3", 1, 3}};
        for (auto &c : cfg) {
            std::unique_ptr<AccumulatorInterface> a = createAccumulator(obs, c.bs, c.skip);
            a->allocate(n);
            WalkerState w(nd, true);
            for (int64_t i = 0; i < n; ++i) {
                std::copy(x.begin() + i * nd, x.begin() + (i + 1) * nd, w.xnew);
                w.nchanged = nd;
                w.accepted = accv[i];
                a->accumulate(w);
            }
            a->finalize();
            put_array(c.name, a->getData(), a->getNData());
        }
    }
    run_file_case();
    // full integrations
    const RunSpec runs[] = {
        // name, nd, seed, move, veclen, pdf, obsset, bs, skip, estim, nfind, ndecorr, nmc, periodic, target, nbits
        {"c1_seed1234", 3, 1234, 0, 0, 0, 0, 1024, 1, (int)EstimatorType::MJBlocker, -50, 1000, 1 << 20, 0, 0.5, 16384},
        {"all_uniform_full", 3, 5649871, 0, 0, 1, 1, 1, 1, -1, 20, 2000, 16384, 0, 0.5, 16384},
        {"all_gauss_block", 3, 1337, 1, 0, 0, 0, 16, 1, -1, 20, 2000, 16384, 0, 0.5, 16384},
        {"vec1_uniform", 3, 1337, 2, 1, 0, 2, 1, 3, -1, -50, 1000, 3 * 8192, 0, 0.5, 16384},
        {"vec3_gauss_nd6", 6, 77, 5, 3, 0, 0, 1, 2, -1, -50, 500, 8192, 0, 0.5, 8192},
        {"typed_all", 3, 1337, 4, 0, 0, 2, 8, 2, -1, -50, 1000, 16384, 0, 0.5, 16384},
        {"multistep_exp", 3, 1337, 3, 0, 0, 2, 1, 1, -1, -50, 500, 8192, 0, 0.85, 8192},
        {"exp_pdf_simple", 4, 31337, 0, 0, 2, 0, 0, 1, -1, -50, 500, 8192, 0, 0.5, 8192},
        {"periodic_3dgauss", 3, 5649871, 0, 0, 1, 1, 1, 1, -1, 10, 1000, 10000, 1, 0.5, 4096},
        {"nopdf_periodic", 3, 5649871, 0, 0, 3, 3, 1, 1, 1, 0, 0, 10000, 1, 0.5, 64},
        {"auto_decorr", 3, 2024, 0, 0, 0, 0, 1, 1, -1, -50, -10000, 8192, 0, 0.5, 8192},
        {"srrd_student_all", 3, 211, 12, 0, 0, 0, 16, 1, -1, -50, 500, 4096, 0, 0.5, 4096},
        {"srrd_cauchy_all", 3, 311, 13, 0, 0, 0, 16, 1, -1, -50, 500, 4096, 0, 0.5, 4096},
        {"srrd_exponential_vec1", 4, 411, 14, 1, 0, 0, 16, 1, -1, -50, 500, 4096, 0, 0.5, 4096},
        {"srrd_gamma_all", 3, 511, 15, 0, 0, 0, 16, 1, -1, -50, 500, 4096, 0, 0.5, 4096},
        {"srrd_weibull_all", 3, 611, 16, 0, 0, 0, 16, 1, -1, -50, 500, 4096, 0, 0.5, 4096},
        {"srrd_lognormal_all", 3, 711, 17, 0, 0, 0, 16, 1, -1, -50, 500, 4096, 0, 0.5, 4096},
        {"srrd_chisq_vec1", 4, 811, 18, 1, 0, 0, 16, 1, -1, -50, 500, 4096, 0, 0.5, 4096},
        {"srrd_fisher_all", 3, 911, 19, 0, 0, 0, 16, 1, -1, -50, 500, 4096, 0, 0.5, 4096},
    };
    const int nruns = sizeof(runs) / sizeof(runs[0]);
    for (int i = 0; i < nruns; ++i) { run_case(runs[i], i == nruns - 1); }
    std::printf("}\n");
    return 0;
}
