// Generated by gen_besselfit.py: polynomial approximations of H0^(2), H1^(2) for FP32
// evaluation (forms of Abramowitz & Stegun 9.4.1-9.4.6, coefficients fitted against
// scipy.special).  Coefficients in ascending powers; x < 3: u = (x/3)^2, x >= 3: t = 3/x.
#pragma once

// max fit error 1.1e-11
#define BGB_BESSEL_P0 {1.000000000e+00f, -2.249999999e+00f, 1.265624970e+00f, -3.164060127e-01f, 4.449369232e-02f, -4.002504988e-03f, 2.478779673e-04f, -9.979368698e-06f}
#define BGB_BESSEL_P0_N 8
// max fit error 1.5e-11
#define BGB_BESSEL_Q0 {3.674669052e-01f, 6.055939492e-01f, -7.435075072e-01f, 2.530200569e-01f, -4.266126158e-02f, 4.346771519e-03f, -2.951379346e-04f, 1.269209462e-05f}
#define BGB_BESSEL_Q0_N 8
// max fit error 7.8e-11
#define BGB_BESSEL_P1 {4.999999999e-01f, -5.624999923e-01f, 2.109373771e-01f, -3.955004019e-02f, 4.447331082e-03f, -3.305473198e-04f, 1.552471554e-05f}
#define BGB_BESSEL_P1_N 7
// max fit error 2.3e-10
#define BGB_BESSEL_Q1 {-6.366197726e-01f, 2.212066146e-01f, 2.168307677e+00f, -1.316686877e+00f, 3.129546586e-01f, -4.090384977e-02f, 3.371409328e-03f, -1.675079926e-04f}
#define BGB_BESSEL_Q1_N 8
// max fit error 2.7e-09
#define BGB_BESSEL_F0 {7.978845635e-01f, -3.675485639e-07f, -5.532674334e-03f, -7.013046538e-05f, 1.315327816e-03f, -6.605469435e-04f, 1.049942381e-04f, 9.179307628e-06f}
#define BGB_BESSEL_F0_N 8
// max fit error 2.0e-09
#define BGB_BESSEL_G0 {-1.514722095e-09f, -4.166649106e-02f, -3.099809436e-06f, 2.428433068e-03f, -1.583243527e-05f, -1.030633675e-03f, 6.580482354e-04f, -1.472100363e-04f}
#define BGB_BESSEL_G0_N 8
// max fit error 4.0e-09
#define BGB_BESSEL_F1 {7.978845568e-01f, 5.383943399e-07f, 1.661071916e-02f, 1.003943391e-04f, -2.321109275e-03f, 9.108218829e-04f, -5.218842491e-05f, -3.879747841e-05f}
#define BGB_BESSEL_F1_N 8
// max fit error 2.3e-09
#define BGB_BESSEL_G1 {1.421697021e-09f, 1.249998475e-01f, 2.283063365e-06f, -6.083108354e-03f, -4.911559033e-05f, 1.916746145e-03f, -1.088043863e-03f, 2.252811010e-04f}
#define BGB_BESSEL_G1_N 8
