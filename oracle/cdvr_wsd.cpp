// cdvr_wsd.cpp -- CPU restatement of the grid step of QuTree's CDVR: the
// multi-matrix branch of LayerGrid (src/DVR/TDDVR.cpp:63-89) around the
// weighted simultaneous diagonalisation
// (src/Util/WeightedSimultaneousDiagonalization.cpp:5-378) and its Jacobi
// rotation helpers (src/Core/JacobiRotationFramework.cpp:4-164).
//
// TEST INFRASTRUCTURE ONLY: loaded by oracle/cdvr.py as the checker of the
// device kernel k_wsd; the product path never links it.
//
// The iteration is discontinuous in its inputs (accept / reject decisions of
// the rational-function optimiser), so this file fixes one operation order
// and the device kernel follows it bit for bit:
//  * a complex product is (ac - bd) + i(ad + bc) (the Givens rotations' real
//    c multiplies both parts alone), sums are left to right and
//    nothing is fused (compiled with -ffp-contract=off; the device file with
//    -fmad=false); a sum over the matrices of a problem is the pairwise tree
//    of the values padded with zeros to a power of two (level by level,
//    t[i] = t[2i] + t[2i+1]); the measure adds its per-matrix traces in
//    index order;
//  * |z| is sqrt(re^2 + im^2) where the reference calls std::abs (hypot), and
//    real(x / w) is (xr wr + xi wi) / (wr^2 + wi^2); the rotated diagonals
//    of a candidate rotation use the Hermitian form (below);
//  * the 3x3 symmetric eigenproblem of the optimiser (Matrix::rDiag, Eigen's
//    SelfAdjointEigenSolver in the reference) is solved for what the
//    optimiser uses of it -- the eigenvector of the largest eigenvalue as
//    ratios v0/v2, v1/v2 and its squared first two components: H is scaled
//    by a power of two (largest |entry| in [1, 2)); the largest root of the
//    characteristic polynomial comes from Newton's method in binary32 from
//    the Gershgorin bound, then Newton's method in binary64, monotone from
//    above, from that root plus 2^-17 (or from the Gershgorin bound when the
//    signs of p, p' and p'' there do not prove it an upper bound), each
//    step's quotient taken in binary32, until a step is below 2^-30; then v
//    is the largest cross product of two rows of H - lambda (absolute
//    accuracy like a rotation method's).  Binary32 values enter and leave
//    by bit operations: truncation of the significand to 23 bits, zero
//    below 2^-126, infinity above the binary32 range;
//  * the two step-size searches stop after 64 rounds at the latest (the
//    reference's own conditions end them far earlier).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

struct cd {
  double r, i;
};
inline cd mk(double r, double i) { return cd{r, i}; }
inline cd cmul(cd a, cd b) { return cd{a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r}; }
inline cd cadd(cd a, cd b) { return cd{a.r + b.r, a.i + b.i}; }
inline cd csub(cd a, cd b) { return cd{a.r - b.r, a.i - b.i}; }
inline cd cconj(cd a) { return cd{a.r, -a.i}; }
inline double cabs_(cd a) { return std::sqrt(a.r * a.r + a.i * a.i); }
inline double cdiv_re(cd x, cd w) { return (x.r * w.r + x.i * w.i) / (w.r * w.r + w.i * w.i); }

constexpr int kMaxMats = 256;

double tree_sum(const double* v, int n) {
  int P = 1;
  while (P < n) P <<= 1;
  double t[kMaxMats];
  for (int i = 0; i < P; ++i) t[i] = i < n ? v[i] : 0.0;
  for (int s = P; s > 1; s >>= 1)
    for (int i = 0; i < s / 2; ++i) t[i] = t[2 * i] + t[2 * i + 1];
  return t[0];
}

struct Mat {
  int d;
  std::vector<cd> a;
  cd& operator()(int i, int j) { return a[i + (size_t)d * j]; }
  cd operator()(int i, int j) const { return a[i + (size_t)d * j]; }
};

// Matrix::rDiag for the optimiser's symmetric 3x3 matrix H: the eigenvector
// v of the largest eigenvalue as the ratios u0 = v0/v2, u1 = v1/v2 and the
// squared norm of its first two components, v0^2 + v1^2 for |v| = 1.
extern "C" void orc_eig3_top(const double H[9], double* u0, double* u1, double* top2);
void eig3_top(const double H[9], double* u0, double* u1, double* top2) { orc_eig3_top(H, u0, u1, top2); }
}  // namespace
// binary64 -> binary32 by truncation of the significand (bit operations, the
// same on every host and on the device); zero below 2^-126, infinity above
static float f32_trunc(double x) {
  uint64_t b;
  std::memcpy(&b, &x, 8);
  const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7ff) - 896;
  uint32_t r;
  if (e <= 0)
    r = sign;
  else if (e >= 255)
    r = sign | 0x7f800000u;
  else
    r = sign | ((uint32_t)e << 23) | (uint32_t)((b >> 29) & 0x7fffffu);
  float f;
  std::memcpy(&f, &r, 4);
  return f;
}
// binary32 -> binary64, exact for normal numbers; subnormals become zero
static double f64_of(float f) {
  uint32_t r;
  std::memcpy(&r, &f, 4);
  const uint64_t sign = (uint64_t)(r & 0x80000000u) << 32;
  const uint32_t e = (r >> 23) & 0xffu;
  uint64_t b;
  if (e == 0)
    b = sign;
  else if (e == 255)
    b = sign | 0x7ff0000000000000ull | ((uint64_t)(r & 0x7fffffu) << 29);
  else
    b = sign | ((uint64_t)(e + 896) << 52) | ((uint64_t)(r & 0x7fffffu) << 29);
  double x;
  std::memcpy(&x, &b, 8);
  return x;
}
extern "C" void orc_eig3_top(const double H[9], double* u0, double* u1, double* top2) {
  double h00 = H[0], h01 = H[3], h02 = H[6], h11 = H[4], h12 = H[7], h22 = H[8];
  // scale by 2^(1023 - e), e the largest biased exponent: max |entry| in [1, 2)
  {
    const double hv[6] = {h00, h01, h02, h11, h12, h22};
    int e = 0;
    for (int i = 0; i < 6; ++i) {
      uint64_t b;
      std::memcpy(&b, &hv[i], 8);
      const int ei = (int)((b >> 52) & 0x7ff);
      if (ei > e) e = ei;
    }
    if (e >= 1 && e <= 2045) {
      const uint64_t sb = (uint64_t)(2046 - e) << 52;
      double sc;
      std::memcpy(&sc, &sb, 8);
      h00 *= sc;
      h01 *= sc;
      h02 *= sc;
      h11 *= sc;
      h12 *= sc;
      h22 *= sc;
    }
  }
  const double tr = h00 + h11 + h22;
  const double m = (h00 * h11 - h01 * h01) + (h00 * h22 - h02 * h02) + (h11 * h22 - h12 * h12);
  const double det = h00 * (h11 * h22 - h12 * h12) - h01 * (h01 * h22 - h12 * h02) + h02 * (h01 * h12 - h11 * h02);
  // Gershgorin upper bound of the largest eigenvalue
  double lam_g = h00 + std::fabs(h01) + std::fabs(h02);
  const double r1 = h11 + std::fabs(h01) + std::fabs(h12);
  const double r2 = h22 + std::fabs(h02) + std::fabs(h12);
  if (r1 > lam_g) lam_g = r1;
  if (r2 > lam_g) lam_g = r2;
  // binary32 Newton from the bound: p(l) = -l^3 + tr l^2 - m l + det
  float fl = f32_trunc(lam_g);
  {
    const float f00 = f32_trunc(h00), f01 = f32_trunc(h01), f02 = f32_trunc(h02);
    const float f11 = f32_trunc(h11), f12 = f32_trunc(h12), f22 = f32_trunc(h22);
    const float ftr = f00 + f11 + f22;
    const float fm = (f00 * f11 - f01 * f01) + (f00 * f22 - f02 * f02) + (f11 * f22 - f12 * f12);
    const float fdet = f00 * (f11 * f22 - f12 * f12) - f01 * (f01 * f22 - f12 * f02) + f02 * (f01 * f12 - f11 * f02);
    for (int it = 0; it < 40; ++it) {
      const float p = ((-fl + ftr) * fl - fm) * fl + fdet;
      const float dp = (-3.0f * fl + 2.0f * ftr) * fl - fm;
      if (!(dp < 0.0f)) break;
      const float nx = fl - p / dp;
      if (!(nx < fl)) break;
      fl = nx;
    }
  }
  // binary64 Newton, monotone from above; p < 0, p' < 0 and p'' < 0 at the
  // start prove it above the largest root
  double lam = f64_of(fl) + 0x1p-17;
  double p = ((-lam + tr) * lam - m) * lam + det;
  double dp = (-3.0 * lam + 2.0 * tr) * lam - m;
  if (!(p < 0.0 && dp < 0.0 && 3.0 * lam > tr)) {
    lam = lam_g;
    p = ((-lam + tr) * lam - m) * lam + det;
    dp = (-3.0 * lam + 2.0 * tr) * lam - m;
  }
  for (int it = 0; it < 100; ++it) {
    if (!(dp < 0.0)) break;
    double step = f64_of(f32_trunc(p) / f32_trunc(dp));
    if (!(std::fabs(step) <= 16.0)) step = p / dp;
    const double nxt = lam - step;
    if (!(nxt < lam)) break;
    lam = nxt;
    if (step <= 0x1p-30) break;
    p = ((-lam + tr) * lam - m) * lam + det;
    dp = (-3.0 * lam + 2.0 * tr) * lam - m;
  }
  // eigenvector: the largest cross product of two rows of H - lambda
  const double m00 = h00 - lam, m11 = h11 - lam, m22 = h22 - lam;
  const double c01[3] = {h01 * h12 - h02 * m11, h02 * h01 - m00 * h12, m00 * m11 - h01 * h01};
  const double c02[3] = {h01 * m22 - h02 * h12, h02 * h02 - m00 * m22, m00 * h12 - h01 * h02};
  const double c12[3] = {m11 * m22 - h12 * h12, h12 * h02 - h01 * m22, h01 * h12 - m11 * h02};
  const double n01 = c01[0] * c01[0] + c01[1] * c01[1] + c01[2] * c01[2];
  const double n02 = c02[0] * c02[0] + c02[1] * c02[1] + c02[2] * c02[2];
  const double n12 = c12[0] * c12[0] + c12[1] * c12[1] + c12[2] * c12[2];
  const double* v = c01;
  double nv = n01;
  if (n02 > nv) {
    v = c02;
    nv = n02;
  }
  if (n12 > nv) {
    v = c12;
    nv = n12;
  }
  *u0 = v[0] / v[2];
  *u1 = v[1] / v[2];
  const double q = v[0] * v[0] + v[1] * v[1];
  *top2 = q / (q + v[2] * v[2]);
}
namespace {

// rotatedDiagonals (src/Core/JacobiRotationFramework.cpp:129-141) for a
// Hermitian A and a real c (the optimiser's c is always real):
//   a0 = c^2 A_pp + 2c Re(s A_pq) + |s|^2 A_qq,  a1 = c^2 A_qq - 2c Re(s A_pq) + |s|^2 A_pp,
// equal to the reference's complex expression up to rounding
inline void rotated_diagonals(const Mat& A, int p, int q, cd c, cd s, double& a0, double& a1) {
  const double cc2 = c.r * c.r;
  const double ss2 = s.r * s.r + s.i * s.i;
  const double c2 = 2.0 * c.r;
  const cd apq = A(p, q);
  const double t = s.r * apq.r - s.i * apq.i;
  const double ct = c2 * t;
  a0 = (cc2 * A(p, p).r + ct) + ss2 * A(q, q).r;
  a1 = (cc2 * A(q, q).r - ct) + ss2 * A(p, p).r;
}

struct Problem {
  int n, d;
  std::vector<Mat> xw;  // weighted matrices
  std::vector<Mat> xp;  // plain (shifted) matrices
  Mat w, trafo;

  // weightedJacobiLoc (WeightedSimultaneousDiagonalization.cpp:260-288)
  double loc(int p, int q, cd c, cd s) const {
    double w0, w1;
    rotated_diagonals(w, p, q, c, s, w0, w1);
    double o0[kMaxMats], o1[kMaxMats], n0[kMaxMats], n1[kMaxMats];
    for (int k = 0; k < n; ++k) {
      const double x0 = xw[k](p, p).r, x1 = xw[k](q, q).r;
      o0[k] = x0 * x0;
      o1[k] = x1 * x1;
    }
    for (int k = 0; k < n; ++k) {
      double r0, r1;
      rotated_diagonals(xw[k], p, q, c, s, r0, r1);
      n0[k] = r0 * r0;
      n1[k] = r1 * r1;
    }
    const double xold0 = tree_sum(o0, n), xold1 = tree_sum(o1, n);
    const double xnew0 = tree_sum(n0, n), xnew1 = tree_sum(n1, n);
    double diff = 0;
    diff += xnew0 / w0 - xold0 / w(p, p).r;
    diff += xnew1 / w1 - xold1 / w(q, q).r;
    return diff;
  }

  // weightedJacobiDerivatives (:290-324)
  void derivatives(double grad[2], double pre[4], cd s_in, int p, int q, double delta) const {
    const double s0 = s_in.r, s1 = s_in.i;
    double y[9];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        const double x0 = s0 + (double)(i - 1) * delta;
        const double x1 = s1 + (double)(j - 1) * delta;
        const double z = x0 * x0 + x1 * x1;
        const cd cnow = mk(std::sqrt(std::fabs(1 - z)), 0.0);
        y[i + 3 * j] = loc(p, q, cnow, mk(x0, x1));
      }
    auto Y = [&](int i, int j) { return y[i + 3 * j]; };
    grad[0] = (Y(2, 1) - Y(0, 1)) / (2 * delta);
    grad[1] = (Y(1, 2) - Y(1, 0)) / (2 * delta);
    pre[0] = (Y(2, 1) + Y(0, 1) - 2 * Y(1, 1)) / (delta * delta);
    pre[3] = (Y(1, 2) + Y(1, 0) - 2 * Y(1, 1)) / (delta * delta);
    pre[2] = (Y(2, 2) + Y(0, 0) - Y(2, 0) - Y(0, 2)) / (4 * delta * delta);
    pre[1] = pre[2];
  }

  // calculateWeightedAngles (:104-211): rational function optimisation
  void angles(cd& c, cd& s, int p, int q) const {
    int iter = 0;
    const int maxiter = 30;
    const double eps = 1E-3;
    double diff_rel = 2 * eps * eps;
    const double amin = 1E-12, amax = 1;
    double a = amax;
    const double delta = 1E-5;
    double snew[2] = {0, 0}, cnew[2] = {0, 0};
    c = mk(std::sqrt(1 - 2 * eps * eps), 0);
    s = mk(eps, -eps);
    double loc_alt = loc(p, q, c, s);
    double loc_new = 0;
    while (iter < maxiter && diff_rel > eps * eps && a > amin) {
      double pre[4], grad[2];
      derivatives(grad, pre, s, p, q, delta);
      double diff = -1;
      int guard = 0;
      while (a > amin && diff < 0 && diff_rel > eps * eps && guard++ < 64) {
        double z = 1;
        double top2 = 0;
        int guard2 = 0;
        while (a > amin && z > 0.5 && guard2++ < 64) {
          // rfoBuildHessian (src/Core/JacobiRotationFramework.cpp:114-127)
          double H[9];
          H[0] = pre[0] * a * a;
          H[1] = pre[1] * a * a;
          H[3] = pre[2] * a * a;
          H[4] = pre[3] * a * a;
          H[2] = grad[0] * a;
          H[6] = grad[0] * a;
          H[5] = grad[1] * a;
          H[7] = grad[1] * a;
          H[8] = 0;
          double u0, u1;
          eig3_top(H, &u0, &u1, &top2);
          const double ds0 = a * u0;
          const double ds1 = a * u1;
          snew[0] = s.r + ds0;
          snew[1] = s.i + ds1;
          const double zab = cabs_(mk(snew[0], snew[1]));
          z = zab * zab;
          if (z > 0.5) a /= 2;
        }
        cnew[0] = std::sqrt(std::fabs(1 - z));
        cnew[1] = 0;
        loc_new = loc(p, q, mk(cnew[0], cnew[1]), mk(snew[0], snew[1]));
        const double trafoabs = top2;
        const double sab = cabs_(s);
        const double sabs = sab * sab + eps * eps;
        diff_rel = trafoabs / sabs;
        diff = loc_new - loc_alt;
        if (diff < 0) {
          a /= 2;
        } else {
          if (a < amax) a *= 2;
        }
      }
      if (a > amin && diff > 0) {
        c = mk(cnew[0], cnew[1]);
        s = mk(snew[0], snew[1]);
        loc_alt = loc_new;
      }
      iter++;
    }
  }

  // givensRotation (src/Core/JacobiRotationFramework.cpp:4-30)
  // c is real (the optimiser's c always is): c x = (c.r x.r, c.r x.i); the
  // full complex product would differ only in the sign of a zero
  static cd rmul(cd c, cd x) { return cd{c.r * x.r, c.r * x.i}; }
  static void givens(Mat& B, cd c, cd s, int i, int j) {
    const int d = B.d;
    std::vector<cd> c0(d), c1(d);
    for (int r = 0; r < d; ++r) {
      c0[r] = cadd(rmul(c, B(r, i)), cmul(s, B(r, j)));
      c1[r] = csub(rmul(c, B(r, j)), cmul(cconj(s), B(r, i)));
    }
    for (int r = 0; r < d; ++r) {
      B(r, i) = c0[r];
      B(r, j) = c1[r];
    }
    for (int r = 0; r < d; ++r) {
      c0[r] = B(i, r);
      c1[r] = B(j, r);
    }
    for (int r = 0; r < d; ++r) {
      B(i, r) = cadd(rmul(c, c0[r]), cmul(cconj(s), c1[r]));
      B(j, r) = csub(rmul(c, c1[r]), cmul(s, c0[r]));
    }
  }

  // givensTrafoRotation (:40-54)
  static void givens_trafo(Mat& T, cd c, cd s, int i, int j) {
    for (int r = 0; r < T.d; ++r) {
      const cd ti = T(r, i), tj = T(r, j);
      T(r, i) = cadd(rmul(c, ti), cmul(s, tj));
      T(r, j) = csub(rmul(c, tj), cmul(cconj(s), ti));
    }
  }

  // weightedJacobiRotations (:75-102)
  void rotations() {
    for (int i = 0; i < d - 1; ++i)
      for (int j = i + 1; j < d; ++j) {
        cd c, s;
        angles(c, s, i, j);
        for (int k = 0; k < n; ++k) givens(xw[k], c, s, i, j);
        givens(w, c, s, i, j);
        givens_trafo(trafo, c, s, i, j);
      }
  }

  // measureWeightedOffDiagonality (:326-353): sum_k Re tr(W (D_k - T^H X_k T)^2)
  double offdiag_one(int k) const {
    std::vector<cd> M(d * d), Y(d * d), Z(d * d);
    const Mat& X = xp[k];
    for (int j = 0; j < d; ++j)  // M = X T
      for (int i = 0; i < d; ++i) {
        cd acc = mk(0, 0);
        for (int l = 0; l < d; ++l) acc = cadd(acc, cmul(X(i, l), trafo(l, j)));
        M[i + d * j] = acc;
      }
    for (int j = 0; j < d; ++j)  // Y = diag(x) - T^H M
      for (int i = 0; i < d; ++i) {
        cd acc = mk(0, 0);
        for (int l = 0; l < d; ++l) acc = cadd(acc, cmul(cconj(trafo(l, i)), M[l + d * j]));
        cd dg = mk(0, 0);
        if (i == j) dg = mk(cdiv_re(xw[k](i, i), w(i, i)), 0);
        Y[i + d * j] = csub(dg, acc);
      }
    for (int j = 0; j < d; ++j)  // Z = Y Y
      for (int i = 0; i < d; ++i) {
        cd acc = mk(0, 0);
        for (int l = 0; l < d; ++l) acc = cadd(acc, cmul(Y[i + d * l], Y[l + d * j]));
        Z[i + d * j] = acc;
      }
    double tr = 0;  // Re tr(W Z)
    for (int i = 0; i < d; ++i) {
      cd acc = mk(0, 0);
      for (int l = 0; l < d; ++l) acc = cadd(acc, cmul(w(i, l), Z[l + d * i]));
      tr += acc.r;
    }
    return tr;
  }
  double offdiag() const {
    double loc = 0;
    for (int k = 0; k < n; ++k) loc += offdiag_one(k);
    return loc;
  }
};

}  // namespace

extern "C" {

// LayerGrid, several matrices (src/DVR/TDDVR.cpp:72-88) with
// WeightedSimultaneousDiagonalization::calculate (:5-53, :369-377):
//   w = regularize(W, 1e-9); shift_k = |tr X_k|; X_k -= shift_k;
//   Xw_k = (X_k w + w X_k) / 2; sweeps of weighted Jacobi rotations until the
//   weighted off-diagonality or its change drops below eps (at most 25);
//   grid_k(i) = Re(Xw_k(i,i) / w(i,i)) + shift_k;  trafo_out = T^dagger.
// X: n matrices d x d (complex128, column-major, interleaved); W: d x d.
// info[0] = sweeps run, info[1] = converged.
int orc_layer_grid(int n, int d, const double* X, const double* W, double eps, double* trafo_out,
                   double* grid, int* info) {
  if (n < 1 || d < 1 || n > kMaxMats) return 1;
  Problem P;
  P.n = n;
  P.d = d;
  P.w.d = d;
  P.w.a.assign((const cd*)W, (const cd*)W + (size_t)d * d);
  for (int i = 0; i < d; ++i) {  // regularize (include/Core/Matrix_Implementation.h:717-725)
    cd& x = P.w(i, i);
    x.r += 1e-9 * std::exp(-cabs_(x) / 1e-9);
  }
  std::vector<double> shift(n);
  P.xp.resize(n);
  for (int k = 0; k < n; ++k) {
    Mat& m = P.xp[k];
    m.d = d;
    m.a.assign((const cd*)X + (size_t)k * d * d, (const cd*)X + (size_t)(k + 1) * d * d);
    cd tr = mk(0, 0);  // calculateShift (src/DVR/TDDVR.cpp:32-39)
    for (int i = 0; i < d; ++i) tr = cadd(tr, m(i, i));
    shift[k] = cabs_(tr);
    for (int i = 0; i < d; ++i) m(i, i).r -= shift[k];
  }
  P.trafo.d = d;
  P.trafo.a.assign((size_t)d * d, mk(0, 0));
  for (int i = 0; i < d; ++i) P.trafo(i, i) = mk(1, 0);
  // weightMatrices (src/Core/JacobiRotationFramework.cpp:104-112): (X W + W X) / 2
  P.xw.resize(n);
  for (int k = 0; k < n; ++k) {
    Mat& o = P.xw[k];
    o.d = d;
    o.a.assign((size_t)d * d, mk(0, 0));
    const Mat& x = P.xp[k];
    for (int j = 0; j < d; ++j)
      for (int i = 0; i < d; ++i) {
        cd xw = mk(0, 0), wx = mk(0, 0);
        for (int l = 0; l < d; ++l) {
          xw = cadd(xw, cmul(x(i, l), P.w(l, j)));
          wx = cadd(wx, cmul(P.w(i, l), x(l, j)));
        }
        const cd sum = cadd(xw, wx);
        o(i, j) = mk(0.5 * sum.r, 0.5 * sum.i);
      }
  }
  double delta = P.offdiag();
  int iter = 0;
  bool converged = false;
  while (!converged && iter < 25) {
    P.rotations();
    const double delta_last = delta;
    delta = P.offdiag();
    const double change = std::fabs(delta_last - delta);
    if (delta < eps || change < eps) converged = true;
    iter++;
  }
  for (int k = 0; k < n; ++k)
    for (int i = 0; i < d; ++i) grid[(size_t)k * d + i] = cdiv_re(P.xw[k](i, i), P.w(i, i)) + shift[k];
  cd* T = (cd*)trafo_out;
  for (int j = 0; j < d; ++j)
    for (int i = 0; i < d; ++i) T[i + (size_t)d * j] = cconj(P.trafo(j, i));
  if (info) {
    info[0] = iter;
    info[1] = converged ? 1 : 0;
  }
  return 0;
}

}  // extern "C"
