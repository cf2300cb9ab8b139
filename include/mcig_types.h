/*
 * mcig_types.h -- enumerations shared by the GB300 integrator's C ABI
 * (include/mcig.h) and by its CPU oracle (oracle/mci_oracle.h).
 *
 * The numeric values of MCIG_MOVE_*, MCIG_SRRD_* and MCIG_EST_* follow the
 * declaration order of the reference's enums, so that a binding can cast the
 * reference enum straight to these integers:
 *   MoveType      include/mci/Factories.hpp:104-109
 *   SRRDType      include/mci/Factories.hpp:115-128
 *   EstimatorType include/mci/Factories.hpp:47-54
 *
 * Sampling functions and observables are device functors selected by a kind
 * code plus a flat parameter vector (doubles).  Each kind names the reference
 * test class whose arithmetic it reproduces, where there is one
 * (test/common/TestMCIFunctions.hpp).
 */
#ifndef MCIG_TYPES_H
#define MCIG_TYPES_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes returned by every mcig_* call */
enum mcig_status {
    MCIG_OK = 0,
    MCIG_ERR_INVALID_ARGUMENT = 1, /* std::invalid_argument in the reference */
    MCIG_ERR_DOMAIN = 2,           /* std::domain_error */
    MCIG_ERR_RUNTIME = 3,          /* std::runtime_error */
    MCIG_ERR_CUDA = 4,             /* a CUDA call failed */
    MCIG_ERR_UNSUPPORTED = 5,      /* option not available on the device path */
    MCIG_ERR_TIMEOUT = 6           /* a bounded device wait ran out */
};

/* MoveType (Factories.hpp:104-109); MCIG_MOVE_USER: a trial move of the attached plugin
 * (mcig_set_user_move), the reference's setTrialMove(std::unique_ptr<TrialMoveInterface>) */
enum mcig_move_type { MCIG_MOVE_ALL = 0, MCIG_MOVE_VEC = 1, MCIG_MOVE_MULTISTEP = 2, MCIG_MOVE_USER = 3 };

/* SRRDType (Factories.hpp:115-128) */
enum mcig_srrd {
    MCIG_SRRD_UNIFORM = 0, MCIG_SRRD_GAUSSIAN = 1, MCIG_SRRD_STUDENT = 2, MCIG_SRRD_CAUCHY = 3,
    MCIG_SRRD_EXPONENTIAL = 4, MCIG_SRRD_GAMMA = 5, MCIG_SRRD_WEIBULL = 6, MCIG_SRRD_LOGNORMAL = 7,
    MCIG_SRRD_CHISQ = 8, MCIG_SRRD_FISHER = 9
};

/* EstimatorType (Factories.hpp:47-54) */
enum mcig_estimator {
    MCIG_EST_NOOP = 0, MCIG_EST_UNCORRELATED = 1, MCIG_EST_CORRELATED = 2,
    MCIG_EST_FCBLOCKER = 3, MCIG_EST_MJBLOCKER = 4
};

/* accumulator chosen from blocksize (Factories.hpp:24-38) */
enum mcig_accumulator { MCIG_ACC_SIMPLE = 0, MCIG_ACC_FULL = 1, MCIG_ACC_BLOCK = 2 };

/* Sampling functions.  Parameters in brackets.
 *  GAUSS_SUM   exp(-sum x_i^2), one proto value       (ThreeDimGaussianPDF, :123-148)
 *  GAUSS       exp(-sum x_i^2), one proto per index   (Gauss, :151-190)
 *  EXP         exp(-sum |x_i|), one proto per index   (ExpNDPDF :219-256, Exp1DPDF :192-217)
 *  GAUSS_PREC  exp(-x^T P x / 2)                      [P, ndim*ndim row-major]
 *  GAUSS_BLOCK exp(-sum_{b0<=i<b1} x_i^2 / (2 w^2))   [b0, b1, w]
 *  GAUSS_MIX   sum_c w_c prod_i N(x_i; m_ci, s_ci)     [ncomp, w[ncomp], m[ncomp*ndim], s[ncomp*ndim]]
 */
enum mcig_pdf_kind {
    MCIG_PDF_GAUSS_SUM = 0, MCIG_PDF_GAUSS = 1, MCIG_PDF_EXP = 2,
    MCIG_PDF_GAUSS_PREC = 3, MCIG_PDF_GAUSS_BLOCK = 4, MCIG_PDF_GAUSS_MIX = 5,
    /* MCIG_PDF_USER + k: the k-th sampling function of the plugin attached to the handle
     * (mcig_set_plugin, include/mcig/plugin.cuh), k < MCIG_MAXUSER */
    MCIG_PDF_USER = 100
};

/* Observables.  Number of values in brackets.
 *  X2SUM    sum x_i^2                 [1]     (X2Sum, :415-433)
 *  XND      x_i                       [ndim]  (XND :335-350, UpdateableXND :352-373, X1D :317-332)
 *  X2       x_i^2                     [ndim]  (X2 :436-462, XYZSquared :297-314)
 *  X2MEAN   sum x_i^2 / ndim          [1]     (XSquared, :260-275 for ndim 3)
 *  CONST    params[0]                 [1]     (Constval, :376-391 with 1.3)
 *  POLYNOM  sum x_i                   [1]     (Polynom, :394-412)
 *  X2BLOCK  sum_{b_k<=i<b_k+1} x_i^2  [nb]    params [nb, b_0 .. b_nb]
 *  GAUSSX2  exp(-r2) r2 / (3 pi^1.5)  [1]     (GaussXSquared, :278-294)
 *  XI       x_i of one index i        [1]     params [i]
 */
enum mcig_obs_kind {
    MCIG_OBS_X2SUM = 0, MCIG_OBS_XND = 1, MCIG_OBS_X2 = 2, MCIG_OBS_X2MEAN = 3,
    MCIG_OBS_CONST = 4, MCIG_OBS_POLYNOM = 5, MCIG_OBS_X2BLOCK = 6, MCIG_OBS_GAUSSX2 = 7, MCIG_OBS_XI = 8,
    MCIG_OBS_LOGPDF = 9, /* log of the product of the sampling functions at the walker (depends on them) */
    /* MCIG_OBS_USER + k: the k-th observable of the attached plugin, k < MCIG_MAXUSER */
    MCIG_OBS_USER = 100
};

/* user functors per plugin and kind (sampling functions, observables) */
#define MCIG_MAXUSER 16

/* arithmetic of the sampling loop on the device */
enum mcig_precision {
    MCIG_PREC_FP64 = 0,        /* reference arithmetic (double, reference operation order) */
    MCIG_PREC_FP32 = 1,        /* float pdf/obs, log-space acceptance, Kahan float sums */
    MCIG_PREC_FP32_ACC64 = 2   /* float pdf/obs, log-space acceptance, double sums */
};

/* where the random numbers come from */
enum mcig_rng { MCIG_RNG_PHILOX = 0, MCIG_RNG_TAPE = 1 };

#ifdef __cplusplus
}
#endif
#endif
