// Modified Bessel functions I0, I1, K0, K1 in FP64 from the polynomial
// approximations of Abramowitz & Stegun, Handbook of Mathematical Functions,
// 9.8.1-9.8.8 (absolute/relative error ~1e-7).  The reference evaluates the
// same published approximations (core/src/numericbase.h:79-175), so the 2.5-D
// primary potentials and mixed boundary coefficients agree to rounding.
#pragma once

namespace ertgb {

// 9.8.1 (|x| < 3.75) and 9.8.2 (|x| >= 3.75), t = x / 3.75
__host__ __device__ inline double as_i0(double x) {
    const double ax = fabs(x);
    if (ax < 3.75) {
        double t = x / 3.75;
        t = t * t;
        return 1.0 + t * (3.5156229 + t * (3.0899424 + t * (1.2067492 + t * (0.2659732 +
               t * (0.0360768 + t * 0.0045813)))));
    }
    const double u = 3.75 / ax;
    return (exp(ax) / sqrt(ax)) * (0.39894228 + u * (0.01328592 + u * (0.00225319 + u * (-0.00157565 +
           u * (0.00916281 + u * (-0.02057706 + u * (0.02635537 + u * (-0.01647633 + u * 0.00392377))))))));
}

// 9.8.3 and 9.8.4
__host__ __device__ inline double as_i1(double x) {
    const double ax = fabs(x);
    double r;
    if (ax < 3.75) {
        double t = x / 3.75;
        t = t * t;
        r = ax * (0.5 + t * (0.87890594 + t * (0.51498869 + t * (0.15084934 + t * (0.02658733 +
            t * (0.00301532 + t * 0.00032411))))));
    } else {
        const double u = 3.75 / ax;
        double s = 0.02282967 + u * (-0.02895312 + u * (0.01787654 - u * 0.00420059));
        s = 0.39894228 + u * (-0.03988024 + u * (-0.00362018 + u * (0.00163801 + u * (-0.01031555 + u * s))));
        r = s * (exp(ax) / sqrt(ax));
    }
    return x < 0.0 ? -r : r;
}

// 9.8.5 (0 < x <= 2) and 9.8.6 (x > 2), y = (x/2)^2 resp. 2/x
__host__ __device__ inline double as_k0(double x) {
    if (x <= 2.0) {
        const double y = x * x / 4.0;
        return (-log(x / 2.0) * as_i0(x)) + (-0.57721566 + y * (0.42278420 + y * (0.23069756 +
               y * (0.03488590 + y * (0.00262698 + y * (0.00010750 + y * 0.0000074))))));
    }
    const double y = 2.0 / x;
    return (exp(-x) / sqrt(x)) * (1.25331414 + y * (-0.07832358 + y * (0.02189568 + y * (-0.01062446 +
           y * (0.00587872 + y * (-0.00251540 + y * 0.00053208))))));
}

// 9.8.7 and 9.8.8
__host__ __device__ inline double as_k1(double x) {
    if (x <= 2.0) {
        const double y = x * x / 4.0;
        return (log(x / 2.0) * as_i1(x)) + (1.0 / x) * (1.0 + y * (0.15443144 + y * (-0.67278579 +
               y * (-0.18156897 + y * (-0.01919402 + y * (-0.00110404 + y * (-0.00004686)))))));
    }
    const double y = 2.0 / x;
    return (exp(-x) / sqrt(x)) * (1.25331414 + y * (0.23498619 + y * (-0.03655620 + y * (0.01504268 +
           y * (-0.00780353 + y * (0.00325614 + y * (-0.00068245)))))));
}

}  // namespace ertgb
