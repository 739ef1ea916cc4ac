// Oguri (2021, arXiv:2106.11464) Table 1: the 44-term cored-steep-ellipsoid
// decomposition of the NFW profile, (a_k, s_k) in units of the scale radius.
// The same published values appear in the reference (JAXtronomy
// LensModel/Profiles/nfw_ellipse_cse.py:15-156, high_accuracy=True) and must be
// identical for parity.
#pragma once

namespace lensgb {

constexpr int CSE_NFW_TERMS = 44;

// (constant memory: every thread of a warp reads the same term at a time)
static __constant__ double kCseNfwA[CSE_NFW_TERMS] = {
    1.648988e-18, 6.274458e-16, 3.646620e-17, 3.459206e-15, 2.457389e-14, 1.059319e-13,
    4.211597e-13, 1.142832e-12, 4.391215e-12, 1.556500e-11, 6.951271e-11, 3.147466e-10,
    1.379109e-09, 3.829778e-09, 1.384858e-08, 5.370951e-08, 1.804384e-07, 5.788608e-07,
    3.205256e-06, 1.102422e-05, 4.093971e-05, 1.282206e-04, 4.575541e-04, 7.995270e-04,
    5.013701e-03, 1.403508e-02, 5.230727e-02, 1.898907e-01, 3.643448e-01, 7.203734e-01,
    1.717667e+00, 2.217566e+00, 3.187447e+00, 8.194898e+00, 1.765210e+01, 1.974319e+01,
    2.783688e+01, 4.482311e+01, 5.598897e+01, 1.426485e+02, 2.279833e+02, 5.401335e+02,
    9.743682e+02, 1.775124e+03,
};

static __constant__ double kCseNfwS[CSE_NFW_TERMS] = {
    1.082411e-06, 8.786566e-06, 3.292868e-06, 1.860019e-05, 3.274231e-05, 6.232485e-05,
    9.256333e-05, 1.546762e-04, 2.097321e-04, 3.391140e-04, 5.178790e-04, 8.636736e-04,
    1.405152e-03, 2.193855e-03, 3.179572e-03, 4.970987e-03, 7.631970e-03, 1.119413e-02,
    1.827267e-02, 2.945251e-02, 4.562723e-02, 6.782509e-02, 1.596987e-01, 1.127751e-01,
    2.169469e-01, 3.423835e-01, 5.194527e-01, 8.623185e-01, 1.382737e+00, 2.034929e+00,
    3.402979e+00, 5.594276e+00, 8.052345e+00, 1.349045e+01, 2.603825e+01, 4.736823e+01,
    6.559320e+01, 1.087932e+02, 1.477673e+02, 2.495341e+02, 4.305999e+02, 7.760206e+02,
    2.143057e+03, 1.935749e+03,
};

}  // namespace lensgb
