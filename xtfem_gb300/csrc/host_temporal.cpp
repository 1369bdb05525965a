// host_temporal.cpp -- temporal side of the space-time discretisation.
//
// The mechanical temporal basis has six functions on a slab [t1, t1+dt]: the
// quadratic Lagrange functions N1..N3 on the nodes t1, t1+dt/2, t1+dt and
// their harmonic enrichments N_{3+a} = N_a (sin w t - sin w t_a).  The
// coefficient matrices are the reference's closed-form slab integrals
// (src/stcoeff.f90:62-356): k = int N' N, m = int N' N'', the jump terms ktn,
// mtn at the slab start and ktn1, mtn1 coupling to the previous slab.  The
// formulas are the published ones and have to be the same expressions; they
// are written out once here.
#include <cmath>

#include "host_sparse.h"

namespace xt {

void stcoeff_m(double t1, double dt, double w, double* k, double* m, double* ktn,
               double* mtn, double* ktn1, double* mtn1)
{
#define K_(i, j) k[((j)-1) * 6 + ((i)-1)]
#define M_(i, j) m[((j)-1) * 6 + ((i)-1)]
#define KT(i, j) ktn[((j)-1) * 6 + ((i)-1)]
#define MT(i, j) mtn[((j)-1) * 6 + ((i)-1)]
#define KT1(i, j) ktn1[((j)-1) * 6 + ((i)-1)]
#define MT1(i, j) mtn1[((j)-1) * 6 + ((i)-1)]
    using std::cos;
    using std::sin;
    for (int e = 0; e < 36; ++e) k[e] = m[e] = ktn[e] = mtn[e] = ktn1[e] = mtn1[e] = 0.0;
    const double d2 = dt * dt, w2 = w * w;
    const double d4w4 = d2 * d2 * w2 * w2;
    const double dw = dt * w, d2w2 = d2 * w2, d3w3 = dt * d2 * w * w2;
    const double s1 = sin(t1 * w), sh = sin((dt / 2. + t1) * w), s3 = sin((dt + t1) * w);
    const double c1 = cos(t1 * w), c3 = cos((dt + t1) * w);
    const double s2t = sin(2. * t1 * w), s2e = sin(2. * (dt + t1) * w);
    const double c2t = cos(2. * t1 * w), c2e = cos(2. * (dt + t1) * w);
    const double cdw = cos(dt * w), sdw = sin(dt * w), cd2t = cos((dt + 2. * t1) * w);

    // stiffness of the complete slab
    // The reference writes these fractions as default-real (single-precision)
    // literals, so their values carry float rounding (src/stcoeff.f90:81-83).
    K_(1, 1) = -0.5; K_(1, 2) = (double)(-2.f / 3.f); K_(1, 3) = (double)(1.f / 6.f);
    K_(1, 4) = (-6. * dw * (-12. + d2w2) * c1 + 24. * dw * c3 + (96. - 26. * d2w2 + d4w4) * s1 +
                2. * (-48. + d2w2) * s3) / (2. * d4w4);
    K_(1, 5) = (2. * (dw * (-84. * c1 - 60. * c3 + dw * (18. * s1 + d2w2 * sh - 6. * s3)) -
                      144. * (s1 - s3))) / (3. * d4w4);
    K_(1, 6) = (120. * dw * c1 - 6. * dw * (-28. + d2w2) * c3 - 18. * (-16. + d2w2) * s1 -
                (288. - 42. * d2w2 + d4w4) * s3) / (6. * d4w4);
    K_(2, 1) = (double)(2.f / 3.f); K_(2, 2) = 0.0; K_(2, 3) = (double)(-2.f / 3.f);
    K_(2, 4) = (-2. * (-6. * dw * (-16. + d2w2) * c1 + 48. * dw * c3 +
                       (-24. + d2w2) * ((-6. + d2w2) * s1 + 6. * s3))) / (3. * d4w4);
    K_(2, 5) = (16. * (6. * dw * c1 + 6. * dw * c3 - (-12. + d2w2) * (s1 - s3))) / d4w4;
    K_(2, 6) = (2. * (-48. * dw * c1 + 6. * dw * (-16. + d2w2) * c3 +
                      (-24. + d2w2) * (6. * s1 + (-6. + d2w2) * s3))) / (3. * d4w4);
    K_(3, 1) = (double)(-1.f / 6.f); K_(3, 2) = (double)(2.f / 3.f); K_(3, 3) = 1. / 2.;
    K_(3, 4) = (-6. * dw * (-28. + d2w2) * c1 + 120. * dw * c3 + (288. - 42. * d2w2 + d4w4) * s1 +
                18. * (-16. + d2w2) * s3) / (6. * d4w4);
    K_(3, 5) = (-2. * (144. * s1 + dw * (60. * c1 + 84. * c3 - 6. * dw * s1 + d3w3 * sh) +
                       18. * (-8. + d2w2) * s3)) / (3. * d4w4);
    K_(3, 6) = (96. * (s1 - s3) + dw * (24. * c1 + (72. - 6. * d2w2) * c3 +
                                        dw * (-2. * s1 + (26. - d2w2) * s3))) / (2. * d4w4);
    K_(4, 1) = -K_(1, 4); K_(4, 2) = -K_(2, 4); K_(4, 3) = -K_(3, 4); K_(4, 4) = 0.;
    K_(4, 5) = (576. - 72. * d2w2 - 4. * d4w4 + 6. * (-96. + 13. * d2w2) * c1 * c1 + 576. * s1 * s1 -
                78. * d2w2 * s1 * s1 + 339. * dw * s2t - 6. * d3w3 * s2t +
                96. * dw * c3 * (5. * s1 - 4. * sh) + 48 * dw * (-16 + d2w2) * c1 * sh -
                1152. * s1 * sh + 240. * d2w2 * s1 * sh - 8. * d4w4 * s1 * sh - 1152. * s1 * s3 +
                48. * d2w2 * s1 * s3 + 1152. * sh * s3 - 48. * d2w2 * sh * s3 - 3. * dw * s2e) /
               (12. * d4w4);
    K_(4, 6) = (-1152. + 72. * d2w2 + 2. * d4w4 + 2. * (576. - 84. * d2w2 + d4w4) * cdw -
                6. * (-96. + 7. * d2w2) * c2t + 576. * c2e - 42. * d2w2 * c2e - 1152. * cd2t +
                168. * d2w2 * cd2t - 2. * d4w4 * cd2t + 672. * dw * sdw - 24. * d3w3 * sdw -
                246. * dw * s2t + 3. * d3w3 * s2t + 246. * dw * s2e - 3. * d3w3 * s2e) /
               (24. * d4w4);
    K_(5, 1) = -K_(1, 5); K_(5, 2) = -K_(2, 5); K_(5, 3) = -K_(3, 5); K_(5, 4) = -K_(4, 5);
    K_(5, 5) = 0.;
    K_(5, 6) = -(-576. + 72. * d2w2 + 4. * d4w4 + (576. - 78. * d2w2) * c3 * c3 - 3. * dw * s2t -
                 384. * dw * c1 * sh + 48. * dw * (-16. + d2w2) * c3 * sh - 1152. * s1 * sh +
                 48. * d2w2 * s1 * sh + 480. * dw * c1 * s3 + 1152. * s1 * s3 - 48. * d2w2 * s1 * s3 +
                 1152. * sh * s3 - 240. * d2w2 * sh * s3 + 8. * d4w4 * sh * s3 - 576. * s3 * s3 +
                 78. * d2w2 * s3 * s3 + 339. * dw * s2e - 6. * d3w3 * s2e) /
               (12. * d4w4);
    K_(6, 1) = -K_(1, 6); K_(6, 2) = -K_(2, 6); K_(6, 3) = -K_(3, 6); K_(6, 4) = -K_(4, 6);
    K_(6, 5) = -K_(5, 6); K_(6, 6) = 0.;

    // mass of the complete slab
    M_(1, 1) = -4. / d2; M_(1, 2) = 8. / d2; M_(1, 3) = -4. / d2;
    M_(1, 4) = (3. * dw * c1 - s1 + s3) / d2;
    M_(1, 5) = (4. * (3. * s1 - 2. * sh - s3)) / d2;
    M_(1, 6) = (dw * c3 - 3. * s1 + 3. * s3) / d2;
    M_(2, 4) = (-4. * (dw * c1 - s1 + s3)) / d2;
    M_(2, 5) = (16. * (-s1 + s3)) / d2;
    M_(2, 6) = (-4. * (dw * c3 - s1 + s3)) / d2;
    M_(3, 1) = 4. / d2; M_(3, 2) = -8. / d2; M_(3, 3) = 4. / d2;
    M_(3, 4) = (dw * c1 - 3. * s1 + 3. * s3) / d2;
    M_(3, 5) = (4. * (s1 + 2. * sh - 3. * s3)) / d2;
    M_(3, 6) = (3. * dw * c3 - s1 + s3) / d2;
    M_(4, 4) = -(-2. + d2w2 + 2. * cdw + (1. + d2w2) * c2t + c2e - 2. * cd2t) / (4. * d2);
    M_(4, 5) = (-8. * dw + 4. * d3w3 + 3. * s2t +
                2. * dw * (4. * cdw + 5. * c2t + 2. * c2e - 4. * cd2t - 3. * dw * s2t) - 3. * s2e) /
               (4. * dt * d2 * w);
    M_(4, 6) = (-16. * dw - 2. * d3w3 + 8. * dw * c1 * c1 - 4. * dw * c3 * c3 - 8. * d2w2 * c3 * s1 +
                16. * dw * s1 * s1 - 6. * s2t + 3. * d2w2 * s2t + 8. * dw * s1 * s3 +
                4. * dw * s3 * s3 + 6. * s2e + d2w2 * s2e) /
               (8. * dt * d2 * w);
    M_(5, 4) = -(4. * d3w3 + 10. * dw * c1 * c1 - 4. * dw * c3 * c3 - 10. * dw * s1 * s1 + 3. * s2t +
                 2. * d2w2 * s2t - 16. * d2w2 * c1 * sh + 16. * dw * s1 * sh - 16. * dw * sh * s3 +
                 4. * dw * s3 * s3 - 3. * s2e) /
               (4. * dt * d2 * w);
    M_(5, 5) = (4. * (c2t - c2e + 2. * cos(((3 * dt) / 2. + 2. * t1) * w) -
                      2. * cos(((dt + 4. * t1) * w) / 2.))) / d2;
    M_(5, 6) = (4. * d3w3 - 4. * dw * c1 * c1 + 10. * dw * c3 * c3 + 4. * dw * s1 * s1 + 3. * s2t +
                16. * d2w2 * c3 * sh - 16. * dw * s1 * sh + 16. * dw * sh * s3 - 10. * dw * s3 * s3 -
                3. * s2e - 2. * d2w2 * s2e) /
               (4. * dt * d2 * w);
    M_(6, 4) = (2. * dw + 2. * d3w3 - 4. * dw * cdw + 4. * dw * c1 * c1 + 2. * dw * c2t +
                4. * dw * c2e + 4. * dw * cd2t + 6. * s2t + d2w2 * s2t - 8. * d2w2 * c1 * s3 -
                6. * s2e + 3. * d2w2 * s2e) /
               (8. * dt * d2 * w);
    M_(6, 5) = (8. * dw - 4. * d3w3 - 3. * s2t + 3. * s2e -
                2. * dw * (4. * cdw + 2. * c2t + 5. * c2e - 4. * cd2t + 3. * dw * s2e)) /
               (4. * dt * d2 * w);
    M_(6, 6) = (-2. + d2w2 + 2. * cdw + c2t + (1. + d2w2) * c2e - 2. * cd2t) / (4. * d2);

    // jump terms at the slab start (+) and coupling to the previous slab (-)
    KT(1, 1) = 1.;
    MT(1, 1) = 9. / d2; MT(1, 2) = -12. / d2; MT(1, 3) = 3. / d2;
    MT(1, 4) = (-3. * w * c1) / dt;
    MT(1, 5) = (12. * (-s1 + sh)) / d2;
    MT(1, 6) = (3. * (s1 - s3)) / d2;
    MT(2, 2) = 16. / d2; MT(2, 3) = -4. / d2;
    MT(2, 4) = (4. * w * c1) / dt;
    MT(2, 5) = (16. * (s1 - sh)) / d2;
    MT(2, 6) = (4. * (-s1 + s3)) / d2;
    MT(3, 3) = 1. / d2;
    MT(3, 4) = -((w * c1) / dt);
    MT(3, 5) = (4. * (-s1 + sh)) / d2;
    MT(3, 6) = (s1 - s3) / d2;
    MT(4, 4) = w2 * c1 * c1;
    MT(4, 5) = (4. * w * c1 * (s1 - sh)) / dt;
    MT(4, 6) = (w * c1 * (-s1 + s3)) / dt;
    MT(5, 5) = (16. * (s1 - sh) * (s1 - sh)) / d2;
    MT(5, 6) = (4. * (s1 - sh) * (-s1 + s3)) / d2;
    MT(6, 6) = (s1 - s3) * (s1 - s3) / d2;
    for (int i = 1; i <= 6; ++i)
        for (int j = 1; j < i; ++j) MT(i, j) = MT(j, i);

    KT1(1, 3) = 1.;
    MT1(1, 1) = -3. / d2; MT1(1, 2) = 12. / d2; MT1(1, 3) = -9 / d2;
    MT1(1, 4) = (-3. * (-s1 + s3)) / d2;
    MT1(1, 5) = (-12. * (sh - s3)) / d2;
    MT1(1, 6) = (-3. * w * c3) / dt;
    MT1(2, 1) = 4. / d2; MT1(2, 2) = -16. / d2; MT1(2, 3) = 12. / d2;
    MT1(2, 4) = (4. * (-s1 + s3)) / d2;
    MT1(2, 5) = (16. * (sh - s3)) / d2;
    MT1(2, 6) = (4. * w * c3) / dt;
    MT1(3, 1) = -1. / d2; MT1(3, 2) = 4. / d2; MT1(3, 3) = -3. / d2;
    MT1(3, 4) = -((-s1 + s3) / d2);
    MT1(3, 5) = (-4. * (sh - s3)) / d2;
    MT1(3, 6) = -((w * c3) / dt);
    MT1(4, 1) = (w * c1) / dt;
    MT1(4, 2) = (-4. * w * c1) / dt;
    MT1(4, 3) = (3. * w * c1) / dt;
    MT1(4, 4) = (w * c1 * (-s1 + s3)) / dt;
    MT1(4, 5) = (4. * w * c1 * (sh - s3)) / dt;
    MT1(4, 6) = w2 * c1 * c3;
    MT1(5, 1) = (4. * (s1 - sh)) / d2;
    MT1(5, 2) = (-16. * (s1 - sh)) / d2;
    MT1(5, 3) = (12. * (s1 - sh)) / d2;
    MT1(5, 4) = (4. * (s1 - sh) * (-s1 + s3)) / d2;
    MT1(5, 5) = (16. * (s1 - sh) * (sh - s3)) / d2;
    MT1(5, 6) = (4. * w * c3 * (s1 - sh)) / dt;
    MT1(6, 1) = (-s1 + s3) / d2;
    MT1(6, 2) = (-4. * (-s1 + s3)) / d2;
    MT1(6, 3) = (3. * (-s1 + s3)) / d2;
    MT1(6, 4) = (-s1 + s3) * (-s1 + s3) / d2;
    MT1(6, 5) = (4. * (sh - s3) * (-s1 + s3)) / d2;
    MT1(6, 6) = (w * c3 * (-s1 + s3)) / dt;
#undef K_
#undef M_
#undef KT
#undef MT
#undef KT1
#undef MT1
}

void stcoeff_t(double dt, double* k, double* m, double* ktn, double* mtn, double* ktn1,
               double* mtn1)
{
    // src/stcoeff.f90:1-60; the reference writes the fractions as
    // single-precision literals, so they carry float rounding.  Column-major.
    const double kk[9] = {(double)(2.f / 15.f), (double)(1.f / 15.f), (double)(-1.f / 30.f),
                          (double)(1.f / 15.f), (double)(8.f / 15.f), (double)(1.f / 15.f),
                          (double)(-1.f / 30.f), (double)(1.f / 15.f), (double)(2.f / 15.f)};
    const double mm[9] = {-.5, (double)(-2.f / 3.f), (double)(1.f / 6.f),
                          (double)(2.f / 3.f), 0., (double)(-2.f / 3.f),
                          (double)(-1.f / 6.f), (double)(2.f / 3.f), .5};
    for (int e = 0; e < 9; ++e) {
        k[e] = kk[e] * dt;
        m[e] = mm[e];
        ktn[e] = mtn[e] = ktn1[e] = mtn1[e] = 0.0;
    }
    mtn[0] = 1.;
    mtn1[6] = 1.;  // (1,3), column-major
}

void getfextc_t(double t1, double dt, double* fextc)
{
    // src/getfextc.f90:9-18: the first three assignments are overwritten
    // by the sinusoidal forms, with the reference's w = 2 * 3.14159 / 24
    using std::cos;
    using std::sin;
    const double w = 2 * 3.14159 / 24;
    const double d2w2 = dt * dt * w * w, dw = dt * w;
    fextc[0] = -((3. * dw * cos(t1 * w) + dw * cos((dt + t1) * w) + 4. * sin(t1 * w) -
                  4. * sin((dt + t1) * w)) / d2w2);
    fextc[1] = (4. * (dw * cos(t1 * w) + dw * cos((dt + t1) * w) + 2. * sin(t1 * w) -
                      2. * sin((dt + t1) * w))) / d2w2;
    fextc[2] = -((dw * cos(t1 * w) + 3. * dw * cos((dt + t1) * w) + 4 * sin(t1 * w) -
                  4. * sin((dt + t1) * w)) / d2w2);
}

void getfextc_m(double t1, double w, double dt, double* fextc, double* fint)
{
    using std::cos;
    using std::sin;
    const double d2w2 = dt * dt * w * w, dw = dt * w;
    fextc[0] = -((3. * dw * cos(t1 * w) + dw * cos((dt + t1) * w) + 4. * sin(t1 * w) -
                  4. * sin((dt + t1) * w)) / d2w2);
    fextc[1] = (4. * (dw * cos(t1 * w) + dw * cos((dt + t1) * w) + 2. * sin(t1 * w) -
                      2. * sin((dt + t1) * w))) / d2w2;
    fextc[2] = -((dw * cos(t1 * w) + 3. * dw * cos((dt + t1) * w) + 4 * sin(t1 * w) -
                  4. * sin((dt + t1) * w)) / d2w2);
    fextc[3] = (16. - 4. * d2w2 + 2. * (-7. + d2w2) * cos(2. * t1 * w) - 2. * cos(2. * (dt + t1) * w) +
                8. * dw * cos((dt + t1) * w) * sin(t1 * w) + 9. * dw * sin(2. * t1 * w) -
                32. * sin(t1 * w) * sin((dt + t1) * w) - dw * sin(2. * (dt + t1) * w)) /
               (8. * d2w2);
    fextc[4] = (-cos(2. * t1 * w) + cos(2. * (dt + t1) * w) + 8. * cos(((dt + 4. * t1) * w) / 2.) -
                8. * cos((3. * dt * w) / 2. + 2. * t1 * w) +
                dw * (sin(2. * t1 * w) + sin(2. * (dt + t1) * w) -
                      4. * (sin(((dt + 4. * t1) * w) / 2.) + sin((3. * dt * w) / 2. + 2. * t1 * w)))) /
               (2. * d2w2);
    fextc[5] = (-16. + 4. * d2w2 + 2. * cos(2. * t1 * w) - 2. * (-7. + d2w2) * cos(2. * (dt + t1) * w) -
                dw * sin(2. * t1 * w) + 8. * (dw * cos(t1 * w) + 4. * sin(t1 * w)) * sin((dt + t1) * w) +
                9. * dw * sin(2. * (dt + t1) * w)) /
               (8. * d2w2);
    fint[0] = -1.;
    fint[1] = 0.;
    fint[2] = 1.;
    fint[3] = 0.;
    fint[4] = 0.;
    fint[5] = -sin(t1 * w) + sin(w * (t1 + dt));
}

void nt_table(int nip, const double* tc, double w, double* Nt)
{
    const double dt = tc[2] - tc[0];
    const double st0 = std::sin(w * tc[0]), st1 = std::sin(w * tc[1]), st2 = std::sin(w * tc[2]);
    for (int i = 0; i < nip; ++i) {
        const double t = tc[0] + (double)i * dt / (double)nip;
        const double n1 = 2.0 * (tc[1] - t) * (tc[2] - t) / (dt * dt);
        const double n2 = -4.0 * (tc[0] - t) * (tc[2] - t) / (dt * dt);
        const double n3 = 2.0 * (tc[0] - t) * (tc[1] - t) / (dt * dt);
        const double swt = std::sin(w * t);
        double* r = Nt + (size_t)i * 6;
        r[0] = n1;
        r[1] = n2;
        r[2] = n3;
        r[3] = n1 * (swt - st0);
        r[4] = n2 * (swt - st1);
        r[5] = n3 * (swt - st2);
    }
}

}  // namespace xt
