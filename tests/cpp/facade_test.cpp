// C++ facade test (mirrors the reference's test/ut4/main.cpp and test/ut2/main.cpp
// checks through mcig::MCI): integrals of exp(-x.x) in 3-D, <x.x/3> = 0.5,
// within 3 sigma; error paths throw the reference's exception types.
#include "mcig/MCIntegrator.hpp"

#include <cmath>
#include <cstdio>
#include <stdexcept>

#define CHECK(c)                                                                 \
    do {                                                                         \
        if (!(c)) { std::printf("FAILED %s (line %d)\n", #c, __LINE__); return 1; } \
    } while (0)

int main()
{
    using namespace mcig;
    const double CORRECT = 0.5;
    {
        MCI mci(3, 256, 0, Precision::FP64);
        mci.setSeed(1337);
        mci.addSamplingFunction(ThreeDimGaussianPDF());
        mci.addObservable(XSquared());
        mci.setNfindMRT2Iterations(20);
        mci.setNdecorrelationSteps(2000);
        double x[3] = {5., -5., 10.};
        mci.setX(x);
        double avg = 0., err = 0.;
        mci.integrate(16384, &avg, &err, true, true); // 2^14: Correlated -> MJBlocker
        std::printf("fp64 MJBlocker: %.6f +- %.6f, acceptance %.3f, step %.4f\n", avg, err, mci.getAcceptanceRate(), mci.getMRT2Step(0));
        CHECK(std::fabs(avg - CORRECT) < 3. * err);
        mci.clearObservables();
        mci.addObservable(XSquared(), 16);
        mci.integrate(16384, &avg, &err, false, false);
        CHECK(std::fabs(avg - CORRECT) < 3. * err);
        mci.clearObservables();
        mci.addObservable(XSquared(), 8, 2, false, EstimatorType::Correlated);
        mci.integrate(16384, &avg, &err, false, false);
        CHECK(std::fabs(avg - CORRECT) < 3. * err);
    }
    {
        MCI mci(3, 1024, 0, Precision::FP32);
        mci.setSeed(5649871);
        mci.addSamplingFunction(Gauss());
        mci.addObservable(XSquared());
        mci.addObservable(X2());
        double avg[4], err[4];
        mci.integrate(8192, avg, err);
        for (int i = 0; i < 4; ++i) { CHECK(std::fabs(avg[i] - CORRECT) < 3.5 * err[i]); }
        std::printf("fp32: %.6f +- %.6f\n", avg[0], err[0]);
    }
    {
        MCI mci(3, 64);
        mci.setIRange(-5., 5.);
        mci.addObservable(GaussXSquared(), 1, 1, false, false);
        double avg, err;
        mci.integrate(10000, &avg, &err, false, false);
        CHECK(std::fabs(avg - CORRECT) < 3.5 * err);
        std::printf("no pdf, periodic box: %.6f +- %.6f\n", avg, err);
    }
    {
        MCI mci(3);
        mci.addObservable(XSquared());
        bool thrown = false;
        double a, e;
        try { mci.integrate(100, &a, &e); } catch (const std::domain_error &) { thrown = true; }
        CHECK(thrown);
        mci.addSamplingFunction(Gauss());
        mci.clearObservables();
        mci.addObservable(XSquared(), 3, 1);
        thrown = false;
        try { mci.integrate(100, &a, &e, false, false); } catch (const std::invalid_argument &) { thrown = true; }
        CHECK(thrown);
        thrown = false;
        try { mci.addObservable(XSquared(), 0, 1, false, true); } catch (const std::invalid_argument &) { thrown = true; }
        CHECK(thrown);
    }
    std::printf("facade ok\n");
    return 0;
}
