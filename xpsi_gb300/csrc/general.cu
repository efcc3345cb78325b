// general.cu -- the general cell-mesh integrator (HotRegion with
// symmetry=False: source parameters that vary from cell to cell), replacing
// xpsi/cellmesh/integrator.pyx:48-667 with the blackbody (hot_BB.pyx:54-98),
// numerical 4-D (hot_Num4D.pyx:248-461), burst blackbody (hot_BB_burst.pyx)
// and Pol_Num2D (hot_Num2D.pyx:187-400) atmospheres and the correction for a
// blackbody elsewhere (:577-592); with `stokes`, also Q and U as
// xpsi/cellmesh/integratorIQU.pyx:76-717 does.
//
// The Stokes integrator's polarisation angle (integratorIQU.pyx:593-596) is
// computed from the variables as the leaf loop leaves them: cos psi and
// sin psi of the last leaf, cos alpha, sin alpha and mu of the last leaf
// within the maximum deflection, and eta, cos xi and the leaf index of the
// last (leaf, mirror) assignment -- one angle per (parallel, image).
//
// Unlike the azimuthally invariant integrator, the atmosphere is evaluated
// per cell at every signal phase: per parallel and image, the leaf profiles
// of the redshift factor Z, mu eta and the geometric factor are splined in
// phase (Steffen, Steffen, Akima periodic) and each radiating cell reads
// them at its shifted phases (:533-592).
//
// Work decomposition:
//   1. general_geometry_kernel, one CTA per parallel: leaf geometry (a thread
//      per leaf, all N_L leaves as the reference's loop runs, :316-420), the
//      sequential visibility state machine that also steps Z and mu eta
//      through invisible intervals (one thread, :421-525), the spline pieces
//      (a thread per interval), then a thread per (cell, phase) evaluates the
//      three splines and stores (Z, mu eta, geometric factor) per entry;
//   2. general_accumulate_kernel, one CTA per (parallel, image): tasks of one
//      phase and 8 energies walk the radiating cells in order and sum
//      cellArea (I norm - correction) x geometric factor (:566-592);
//   3. general_reduce_kernel adds the (parallel, image) partials in order and
//      divides by E keV (:600-610).
//
// Num4D call history (hot_Num4D.pyx:300-351): entries are visited in the
// reference's single-thread call order (parallel, image, cell, phase,
// energy).  An evaluation's clamp depends on the previous call's coordinates
// only when a coordinate lies outside the table; that previous call is the
// same entry at the previous energy, or, for the first energy, the last
// entry before it with a positive geometric factor (found by a backward scan
// over the stored entries, only when it is needed).
#include "common.cuh"
#include "kernels.h"
#include "num4d_walk.cuh"

namespace xg {

namespace {

constexpr int kGenThreads = 128;
constexpr int kGenAccThreads = 256;
constexpr int kGenEPT = 8;        // energies per accumulation task
constexpr int kGenWrapLimit = 1024;

struct GenRow {
  const double *D, *CA, *LG;
  int N_R, jalt;
  double Grav_z, cos_gamma, sin_gamma, cos_th, sin_th, th_over_pi, beta, Lorentz, maxDefl;
};

struct GenSmem {
  double *rD;                      // [N_R] staged deflections
  // per leaf, the polarisation angle's inputs as the leaf loop assigns them
  double *xcpsi, *xspsi, *xca, *xsa, *xmu, *xeta, *xcxi;  // [N_L]
  int *xvis, *xks;                 // [N_L] within max deflection; last mirror pass
                                   // (0 none, 1 the leaf, 2 its mirror)
  double *lPH, *lZ, *lAB, *lGE;    // [N_L] leaf values written by the geometry
  double *PH, *ZZ, *AB, *GE;       // [N_L] the state machine's knots and values
  double *pZ, *pA, *pG;            // [4 (N_L - 1)] spline pieces (y, k1, k2, k3)
  int *calc, *term;                // [N_L]
  int *flags;                      // [0] terminate, [1] no visibility
};

__device__ GenSmem gen_carve(double *sm, int N_R, int N_L) {
  GenSmem g;
  g.rD = sm;
  g.lPH = g.rD + N_R;
  g.lZ = g.lPH + N_L;
  g.lAB = g.lZ + N_L;
  g.lGE = g.lAB + N_L;
  g.PH = g.lGE + N_L;
  g.ZZ = g.PH + N_L;
  g.AB = g.ZZ + N_L;
  g.GE = g.AB + N_L;
  g.pZ = g.GE + N_L;
  g.pA = g.pZ + 4 * N_L;
  g.pG = g.pA + 4 * N_L;
  g.xcpsi = g.pG + 4 * N_L;
  g.xspsi = g.xcpsi + N_L;
  g.xca = g.xspsi + N_L;
  g.xsa = g.xca + N_L;
  g.xmu = g.xsa + N_L;
  g.xeta = g.xmu + N_L;
  g.xcxi = g.xeta + N_L;
  g.calc = reinterpret_cast<int *>(g.xcxi + N_L);
  g.term = g.calc + N_L;
  g.xvis = g.term + N_L;
  g.xks = g.xvis + N_L;
  g.flags = g.xks + N_L;
  return g;
}

// one leaf of :316-420: visibility and, for the first half of the leaves,
// the geometry of the leaf and its mirror
__device__ void gen_leaf(const GenRow &r, double cos_i, double sin_i, double incl, int I, int k,
                         int N_L, int leaf_lim, const double *leaves, GenSmem &g) {
  double cos_psi = cos_i * r.cos_th + sin_i * r.sin_th * cos(leaves[k]);
  double psi = image_deflection(I, acos(cos_psi));
  double sin_psi = sin(psi);
  if (!are_equal(psi, 0.0) && are_equal(sin_psi, 0.0)) {
    const double _i = (cos_i >= 0.0) ? incl + incl * 1.0e-6 : incl - incl * 1.0e-6;
    cos_psi = cos(_i) * r.cos_th + sin(_i) * r.sin_th * cos(leaves[k]);
    psi = image_deflection(I, acos(cos_psi));
    sin_psi = sin(psi);
  }
  MainX mx{r.D};
  AltX ax{r.D, r.jalt};
  AltY ay{r.CA, r.jalt};
  const double alt_xmin = cos(r.D[r.jalt]);
  int calc = 0, term = 0, vis = 0, ks_last = 0;
  double sin_alpha = 0.0, mu = 0.0, cos_a = 0.0, eta_last = 0.0, cxi_last = 0.0;
  if (psi <= r.maxDefl) {
    if (psi < r.D[0] || psi > r.D[r.N_R - 1]) {
      term = 1;
    } else {
      vis = 1;
      if (psi <= kHalfPi && cos_psi >= alt_xmin)
        steffen_eval(ax, ay, r.jalt + 1, cos_psi, &cos_a, nullptr);
      else
        steffen_eval(mx, ArrY{r.CA}, r.N_R, psi, &cos_a, nullptr);
      sin_alpha = sqrt(1.0 - cos_a * cos_a);
      mu = cos_a * r.cos_gamma;
      if (!are_equal(psi, 0.0)) {
        const double cos_delta = (cos_i - r.cos_th * cos_psi) / (r.sin_th * sin_psi);
        if (r.th_over_pi < 0.5) mu = mu + sin_alpha * r.sin_gamma * cos_delta;
        else mu = mu - sin_alpha * r.sin_gamma * cos_delta;
      }
      calc = (mu > 0.0) ? 1 : 0;
    }
  }
  if (calc && !term && k < leaf_lim) {
    double deriv;
    if (psi <= kHalfPi && cos_psi >= alt_xmin) {
      steffen_eval(ax, ay, r.jalt + 1, cos_psi, nullptr, &deriv);
    } else {
      steffen_eval(mx, ArrY{r.CA}, r.N_R, psi, nullptr, &deriv);
      deriv = exp(log(fabs(deriv)) - log(fabs(sin_psi)));
    }
    double plag;
    steffen_eval(mx, ArrY{r.LG}, r.N_R, psi, &plag, nullptr);
    for (int ks = 0; ks < 2; ks++) {
      if ((0 < k && k < leaf_lim - 1) || (k == 0 && ks == 0) ||
          (k == leaf_lim - 1 && N_L % 2 == 1 && ks == 0) ||
          (k == leaf_lim - 1 && N_L % 2 == 0)) {
        const int kdx = (ks == 0) ? k : N_L - 1 - k;
        double superlum, eta, cos_xi;
        if (!are_equal(psi, 0.0)) {
          cos_xi = sin_alpha * sin_i * sin(leaves[kdx]) / sin_psi;
          superlum = 1.0 + r.beta * cos_xi;
          eta = r.Lorentz / superlum;
        } else {
          cos_xi = 0.0;
          superlum = 1.0;
          eta = r.Lorentz;
        }
        ks_last = ks + 1;
        eta_last = eta;
        cxi_last = cos_xi;
        g.lZ[kdx] = eta * r.Grav_z;
        g.lAB[kdx] = mu * eta;
        g.lGE[kdx] = mu * fabs(deriv) * r.Grav_z * eta * eta * eta / superlum;
        g.lPH[kdx] = leaves[kdx] + plag;
      }
    }
  }
  g.calc[k] = calc;
  g.term[k] = term;
  g.xcpsi[k] = cos_psi;
  g.xspsi[k] = sin_psi;
  g.xvis[k] = vis;
  g.xca[k] = cos_a;
  g.xsa[k] = sin_alpha;
  g.xmu[k] = mu;
  g.xks[k] = ks_last;
  g.xeta[k] = eta_last;
  g.xcxi[k] = cxi_last;
}

// :421-535, one thread, in the reference's leaf order: a visible leaf's
// values are copied in when the loop reaches it, invisible intervals are
// stepped linearly (phase, Z, mu eta) with a zero geometric factor
__device__ void gen_state_machine(int N_L, int leaf_lim, const double *leaves, GenSmem &g) {
  int InvisFlag = 2, InvisPhase = 0, term = 0;
  double step, Zs, As;
  double *PH = g.PH, *ZZ = g.ZZ, *AB = g.AB, *GE = g.GE;
  for (int k = 0; k < N_L; k++) {
    if (g.term[k]) { term = 1; break; }
    if (g.calc[k]) {
      for (int ks = 0; ks < 2; ks++) {
        if ((0 < k && k < leaf_lim - 1) || (k == 0 && ks == 0) ||
            (k == leaf_lim - 1 && N_L % 2 == 1 && ks == 0) ||
            (k == leaf_lim - 1 && N_L % 2 == 0)) {
          const int kdx = (ks == 0) ? k : N_L - 1 - k;
          PH[kdx] = g.lPH[kdx];
          ZZ[kdx] = g.lZ[kdx];
          AB[kdx] = g.lAB[kdx];
          GE[kdx] = g.lGE[kdx];
        }
      }
      if (k == 0) {
        PH[N_L - 1] = PH[0] + kTwoPi;
        ZZ[N_L - 1] = ZZ[0];
        AB[N_L - 1] = AB[0];
        GE[N_L - 1] = GE[0];
      } else if (k > 0 && InvisFlag == 2) {
        step = leaves[k] / (double)k;
        Zs = (ZZ[k] - ZZ[N_L - k - 1]) / (2.0 * (double)k);
        As = (AB[k] - AB[N_L - k - 1]) / (2.0 * (double)k);
        for (int m = N_L - k; m < N_L; m++) {
          PH[m] = PH[m - 1] + step;
          ZZ[m] = ZZ[m - 1] + Zs;
          AB[m] = AB[m - 1] + As;
          GE[m] = 0.0;
        }
        PH[0] = PH[N_L - 1] - kTwoPi;
        ZZ[0] = ZZ[N_L - 1];
        AB[0] = AB[N_L - 1];
        GE[0] = GE[N_L - 1];
        for (int m = 1; m < k; m++) {
          PH[m] = PH[m - 1] + step;
          ZZ[m] = ZZ[m - 1] + Zs;
          AB[m] = AB[m - 1] + As;
          GE[m] = 0.0;
        }
      } else if (InvisFlag == 1) {
        const double n = (double)(k - InvisPhase + 1);
        step = (PH[k] - PH[InvisPhase - 1]) / n;
        Zs = (ZZ[k] - ZZ[InvisPhase - 1]) / n;
        As = (AB[k] - AB[InvisPhase - 1]) / n;
        for (int m = InvisPhase; m < k; m++) {
          PH[m] = PH[m - 1] + step;
          ZZ[m] = ZZ[m - 1] + Zs;
          AB[m] = AB[m - 1] + As;
        }
        step = (PH[N_L - InvisPhase] - PH[N_L - 1 - k]) / n;
        Zs = (ZZ[N_L - InvisPhase] - ZZ[N_L - 1 - k]) / n;
        As = (AB[N_L - InvisPhase] - AB[N_L - 1 - k]) / n;
        for (int m = N_L - k; m < N_L - InvisPhase; m++) {
          PH[m] = PH[m - 1] + step;
          ZZ[m] = ZZ[m - 1] + Zs;
          AB[m] = AB[m - 1] + As;
        }
      }
      InvisFlag = 0;
    } else if (InvisFlag == 0) {
      const double n = (double)(N_L - 2 * k + 1);
      step = (PH[N_L - k] - PH[k - 1]) / n;
      Zs = (ZZ[N_L - k] - ZZ[k - 1]) / n;
      As = (AB[N_L - k] - AB[k - 1]) / n;
      for (int m = k; m < N_L - k; m++) {
        PH[m] = PH[m - 1] + step;
        ZZ[m] = ZZ[m - 1] + Zs;
        AB[m] = AB[m - 1] + As;
        GE[m] = 0.0;
      }
      InvisFlag = 1;
      InvisPhase = k;
    }
  }
  int invis = 0;
  if (!term) {
    if (InvisFlag == 2) {
      invis = 1;
    } else {
      for (int m = 1; m < N_L; m++)
        if (PH[m] <= PH[m - 1]) { term = 1; break; }
    }
  }
  g.flags[0] = term;
  g.flags[1] = invis;
}

struct SmemX {
  const double *x;
  __device__ double operator()(int j) const { return x[j]; }
};

__global__ void __launch_bounds__(kGenThreads) general_geometry_kernel(GeneralArgs a) {
  const int i = blockIdx.x;
  const int S1 = a.S1, N_R = a.N_R, N_L = a.N_L, N_P = a.N_P;
  const int leaf_lim = (N_L % 2 == 0) ? N_L / 2 : (N_L + 1) / 2;
  extern __shared__ double sm[];
  GenSmem g = gen_carve(sm, N_R, N_L);
  __shared__ int s_J, s_jalt, s_term;
  const int32_t *rad = a.radiates + (int64_t)i * S1;
  if (threadIdx.x == 0) {
    int J = S1;
    for (int j = 0; j < S1; j++)
      if (rad[j] == 1) { J = j; break; }
    s_J = J;
    s_jalt = N_R - 1;
    s_term = 0;
  }
  __syncthreads();
  if (s_J >= S1) {
    if (threadIdx.x == 0) a.n_img[i] = 0;
    return;
  }
  const double *Dg = a.deflection + (int64_t)i * N_R;
  for (int t = threadIdx.x; t < N_R; t += blockDim.x) {
    g.rD[t] = Dg[t];
    if (Dg[t] > kHalfPi) atomicMin(&s_jalt, t);
  }
  __syncthreads();
  GenRow r;
  r.D = g.rD;
  r.CA = a.cos_alpha + (int64_t)i * N_R;
  r.LG = a.lag + (int64_t)i * N_R;
  r.N_R = N_R;
  r.jalt = s_jalt < 1 ? 1 : s_jalt;
  r.Grav_z = sqrt(1.0 - a.u[i]);
  r.cos_gamma = a.cos_gamma[i];
  r.sin_gamma = sqrt(1.0 - r.cos_gamma * r.cos_gamma);
  const double th = a.theta0[i];
  r.cos_th = cos(th);
  r.sin_th = sin(th);
  r.th_over_pi = th / kPi;
  r.beta = a.radius[i] * a.omega * r.sin_th / (kC * r.Grav_z);
  r.Lorentz = sqrt(1.0 - r.beta * r.beta);
  r.maxDefl = a.maxDeflection[i];
  const int IO = a.image_order_limit > 0 ? a.image_order_limit : (int)ceil(r.maxDefl / kPi);
  const double cos_i = cos(a.inclination), sin_i = sin(a.inclination);
  // the polarisation angle's inputs carried over images (thread 0); at the
  // parallel's start cos alpha is -1 (integratorIQU.pyx:326) and the others
  // are not yet assigned
  double x_cpsi = NAN, x_spsi = NAN, x_ca = -1.0, x_sa = NAN, x_mu = NAN, x_eta = NAN,
         x_cxi = NAN;
  int x_kdx = 0;
  int done = 0;
  for (int I = 0; I < IO; I++) {
    if (I >= a.IOmax) {  // more images than the scratch holds
      if (threadIdx.x == 0) atomicExch(a.status, (int)kBadInput);
      break;
    }
    for (int k = threadIdx.x; k < N_L; k += blockDim.x)
      gen_leaf(r, cos_i, sin_i, a.inclination, I, k, N_L, leaf_lim, a.leaves, g);
    __syncthreads();
    if (threadIdx.x == 0) gen_state_machine(N_L, leaf_lim, a.leaves, g);
    __syncthreads();
    if (g.flags[0]) {
      if (threadIdx.x == 0) atomicExch(a.status, (int)kPulseFail);
      break;
    }
    if (g.flags[1]) break;
    if (a.stokes && threadIdx.x == 0) {
      for (int k = 0; k < N_L; k++) {
        x_cpsi = g.xcpsi[k];
        x_spsi = g.xspsi[k];
        if (g.xvis[k]) {
          x_ca = g.xca[k];
          x_sa = g.xsa[k];
          x_mu = g.xmu[k];
        }
        if (g.xks[k]) {
          x_kdx = g.xks[k] == 1 ? k : N_L - 1 - k;
          x_eta = g.xeta[k];
          x_cxi = g.xcxi[k];
        }
      }
      const double chi = pol_angle(a.leaves[x_kdx], x_spsi, x_cpsi, x_sa, x_ca, r.sin_th,
                                   r.cos_th, sin_i, cos_i, r.sin_gamma, r.cos_gamma, r.Grav_z,
                                   x_mu, x_eta, r.beta, r.Lorentz, x_cxi);
      double *c2 = a.chi2 + ((int64_t)i * a.IOmax + I) * 2;
      c2[0] = cos(2 * chi);
      c2[1] = sin(2 * chi);
    }
    // spline pieces: Steffen for Z and mu eta, Akima periodic for the
    // geometric factor (the reference's default phase interpolant)
    for (int t = threadIdx.x; t < N_L - 1; t += blockDim.x) {
      const SmemX X{g.PH};
      const Cubic cz = steffen_piece(X, SmemX{g.ZZ}, N_L, t);
      const Cubic ca = steffen_piece(X, SmemX{g.AB}, N_L, t);
      g.pZ[4 * t] = cz.y0; g.pZ[4 * t + 1] = cz.k1; g.pZ[4 * t + 2] = cz.k2;
      g.pZ[4 * t + 3] = cz.k3;
      g.pA[4 * t] = ca.y0; g.pA[4 * t + 1] = ca.k1; g.pA[4 * t + 2] = ca.k2;
      g.pA[4 * t + 3] = ca.k3;
      auto chord = [&](int j) -> double {
        const int q = periodic_chord(j, N_L);
        return (g.GE[q + 1] - g.GE[q]) / (g.PH[q + 1] - g.PH[q]);
      };
      double k1, k2, k3;
      akima_piece(chord(t - 2), chord(t - 1), chord(t), chord(t + 1), chord(t + 2),
                  g.PH[t + 1] - g.PH[t], k1, k2, k3);
      g.pG[4 * t] = g.GE[t]; g.pG[4 * t + 1] = k1; g.pG[4 * t + 2] = k2; g.pG[4 * t + 3] = k3;
    }
    __syncthreads();
    // the three splines at every (cell, phase) entry (:549-571)
    const int64_t base = ((int64_t)i * a.IOmax + I) * S1 * N_P;
    const double x_lo = g.PH[0], x_hi = g.PH[N_L - 1];
    for (int t = threadIdx.x; t < S1 * N_P; t += blockDim.x) {
      const int j = t / N_P, k = t - j * N_P;
      double G = 0.0, Z = 0.0, A = 0.0;
      if (rad[j] == 1) {
        double x = a.phases[k] + a.phi[(int64_t)i * S1 + j];
        if (x > x_hi) {
          for (int w = 0; x > x_hi && w < kGenWrapLimit; w++) x = x - kTwoPi;
        } else if (x < x_lo) {
          for (int w = 0; x < x_lo && w < kGenWrapLimit; w++) x = x + kTwoPi;
        }
        if (!(x >= x_lo && x <= x_hi)) {
          s_term = 1;
        } else {
          const int iv = locate(g.PH, N_L, x);
          const double u = x - g.PH[iv];
          const double *q = g.pG + 4 * iv;
          G = q[0] + u * (q[1] + u * (q[2] + u * q[3]));
          if (G > 0.0) {
            const double *qz = g.pZ + 4 * iv, *qa = g.pA + 4 * iv;
            Z = qz[0] + u * (qz[1] + u * (qz[2] + u * qz[3]));
            A = qa[0] + u * (qa[1] + u * (qa[2] + u * qa[3]));
          }
        }
      }
      a.eG[base + t] = G;
      a.eZ[base + t] = Z;
      a.eA[base + t] = A;
    }
    __syncthreads();
    if (s_term) {
      if (threadIdx.x == 0) atomicExch(a.status, (int)kPulseFail);
      break;
    }
    done = I + 1;
  }
  if (threadIdx.x == 0) a.n_img[i] = done;
}

// the coordinates of the call before entry t's first energy: the last entry
// before t (in call order) with a positive geometric factor, at the last
// energy; -inf (a fresh walk) when there is none.  Num4D: (log T, log g, mu,
// log10(E/E_eff)); Pol_Num2D: (mu, log10 E) in vp[0..1]
__device__ void gen_prev_coords(const GeneralArgs &a, int64_t t, double vp[4]) {
  const int64_t per_img = (int64_t)a.S1 * a.N_P;
  int64_t u = t - 1;
  while (u >= 0) {
    const int64_t rj = u / per_img;
    const int row = (int)(rj / a.IOmax), I = (int)(rj - (int64_t)row * a.IOmax);
    if (I >= a.n_img[row]) {  // an image the reference never evaluated
      u = rj * per_img - 1;
      continue;
    }
    if (a.eG[u] > 0.0) break;
    u--;
  }
  if (u < 0) {
    vp[0] = vp[1] = vp[2] = vp[3] = -INFINITY;
    return;
  }
  const int64_t rj = u / per_img;
  const int row = (int)(rj / a.IOmax);
  const int j = (int)((u - rj * per_img) / a.N_P);
  if (a.atm_ext == 4) {
    vp[0] = a.eA[u];
    vp[1] = log10(a.energies[a.N_E - 1] / a.eZ[u]);
    vp[2] = vp[3] = 0.0;
    return;
  }
  const double *vec = a.params + ((int64_t)row * a.S1 + j) * a.n_params;
  const double E_eff = (kKB / kKeV) * pow(10.0, vec[0]);
  vp[0] = vec[0];
  vp[1] = vec[1];
  vp[2] = a.eA[u];
  vp[3] = log10((a.energies[a.N_E - 1] / a.eZ[u]) / E_eff);
}

// Pol_Num2D (hot_Num2D.pyx:187-347): the cached walk on (mu, log10 E) after
// a call at vp[2]; the stencil sum without the positive part
__device__ double num2d_walk(const Atmos4D &A, const double *table, const double vp[2],
                             double v0, double v1) {
  double v[2] = {v0, v1};
  const double *g[2] = {A.mu, A.logE};
  const int n[2] = {A.nmu, A.nE};
  int b[2];
  double w[2][4];
#pragma unroll
  for (int d = 0; d < 2; d++) {
    b[d] = walk_base(g[d], n[d], vp[d], v[d]);
    lagrange4(g[d], b[d], v[d], w[d]);
  }
  double I = 0.0;
  for (int i = 0; i < 4; i++) {
    const double *r = table + (size_t)(b[0] + i) * A.nE + b[1];
    I += w[0][i] * (w[1][0] * __ldg(r) + w[1][1] * __ldg(r + 1) + w[1][2] * __ldg(r + 2) +
                    w[1][3] * __ldg(r + 3));
  }
  return I;
}

__global__ void __launch_bounds__(kGenAccThreads) general_accumulate_kernel(GeneralArgs a) {
  const int64_t ri = blockIdx.x;
  const int i = (int)(ri / a.IOmax), I = (int)(ri - (int64_t)i * a.IOmax);
  if (I >= a.n_img[i]) return;
  const int S1 = a.S1, N_P = a.N_P, N_E = a.N_E;
  const bool num4d = a.atm_ext == 2, burst = a.atm_ext == 3, num2d = a.atm_ext == 4;
  const bool stokes = a.stokes != 0;
  const bool corr = a.correction != nullptr;
  const double norm = (num4d || num2d) ? kErg / kHKeV : kErg * kPlanck;
  const double c2chi = stokes ? a.chi2[ri * 2] : 0.0, s2chi = stokes ? a.chi2[ri * 2 + 1] : 0.0;
  extern __shared__ double sm[];
  double *cT = sm, *cC = sm + S1;  // per cell: kT or E_eff; the correction's kT
  for (int j = threadIdx.x; j < S1; j += blockDim.x) {
    const double *vec = a.params + ((int64_t)i * S1 + j) * a.n_params;
    cT[j] = (kKB / kKeV) * pow(10.0, vec[0]);
    cC[j] = corr ? (kKB / kKeV) * pow(10.0, a.correction[((int64_t)i * S1 + j) * a.n_correction])
                 : 0.0;
  }
  __syncthreads();
  const int64_t base = ri * S1 * N_P;
  const int groups = (N_E + kGenEPT - 1) / kGenEPT;
  const int32_t *rad = a.radiates + (int64_t)i * S1;
  const double *cellA = a.cellArea + (int64_t)i * S1;
  for (int task = threadIdx.x; task < N_P * groups; task += blockDim.x) {
    const int k = task % N_P, grp = task / N_P;
    const int p0 = grp * kGenEPT;
    double acc[kGenEPT], accQ[kGenEPT], accU[kGenEPT];
#pragma unroll
    for (int e = 0; e < kGenEPT; e++) acc[e] = accQ[e] = accU[e] = 0.0;
    for (int j = 0; j < S1; j++) {
      if (rad[j] != 1) continue;
      const int64_t t = base + (int64_t)j * N_P + k;
      const double G = a.eG[t];
      if (!(G > 0.0)) continue;
      const double Z = a.eZ[t], AB = a.eA[t], A = cellA[j];
      const double *vec = a.params + ((int64_t)i * S1 + j) * a.n_params;
#pragma unroll
      for (int e = 0; e < kGenEPT; e++) {
        const int p = p0 + e;
        if (p >= N_E) break;
        const double Ep = a.energies[p] / Z;
        double I_E, Q_E = 0.0;
        if (num2d) {
          const double v1 = log10(Ep);
          double vp[4];
          if (p > 0) {
            vp[0] = AB;
            vp[1] = log10(a.energies[p - 1] / Z);
          } else {
            const Atmos4D &T = a.atmos;
            const bool inside = AB >= T.mu[0] && AB <= T.mu[T.nmu - 1] && v1 >= T.logE[0] &&
                                v1 <= T.logE[T.nE - 1];
            if (inside) vp[0] = vp[1] = 0.0;  // not read inside the table
            else gen_prev_coords(a, t, vp);
          }
          I_E = num2d_walk(a.atmos, a.atmos.I, vp, AB, v1);
          if (I_E < 0.0) I_E = 0.0;
          if (stokes && a.table_q) Q_E = num2d_walk(a.atmos, a.table_q, vp, AB, v1);
        } else if (num4d) {
          const double v3 = log10(Ep / cT[j]);
          double vp[4];
          if (p > 0) {
            vp[0] = vec[0];
            vp[1] = vec[1];
            vp[2] = AB;
            vp[3] = log10((a.energies[p - 1] / Z) / cT[j]);
          } else {
            const Atmos4D &T = a.atmos;
            const bool inside = vec[0] >= T.logT[0] && vec[0] <= T.logT[T.nT - 1] &&
                                vec[1] >= T.logg[0] && vec[1] <= T.logg[T.ng - 1] &&
                                AB >= T.mu[0] && AB <= T.mu[T.nmu - 1] &&
                                v3 >= T.logE[0] && v3 <= T.logE[T.nE - 1];
            if (inside) vp[0] = vp[1] = vp[2] = vp[3] = 0.0;  // not read inside the table
            else gen_prev_coords(a, t, vp);
          }
          I_E = num4d_walk(a.atmos, vp, vec[0], vec[1], AB, v3);
        } else if (burst) {  // hot_BB_burst.pyx
          I_E = eval_bb(Ep, cT[j]) * (0.421 + 0.868 * AB);
          Q_E = (0.1171 * (AB - 1.) / (1. + 3.582 * AB)) * I_E;
        } else {
          I_E = eval_bb(Ep, cT[j]);
        }
        I_E = I_E * norm;
        const double c = corr ? eval_bb(Ep, cC[j]) * (kErg * kPlanck) : 0.0;
        acc[e] += A * (I_E - c) * G;
        if (stokes) {  // integratorIQU.pyx:615-633
          Q_E = Q_E * norm;
          accQ[e] += A * (Q_E * c2chi) * G;
          accU[e] += A * (Q_E * s2chi) * G;
        }
      }
    }
    double *part = a.partial + ri * (int64_t)(stokes ? 3 : 1) * N_E * N_P;
#pragma unroll
    for (int e = 0; e < kGenEPT; e++) {
      const int p = p0 + e;
      if (p < N_E) {
        part[(int64_t)p * N_P + k] = acc[e];
        if (stokes) {
          part[(int64_t)(N_E + p) * N_P + k] = accQ[e];
          part[(int64_t)(2 * N_E + p) * N_P + k] = accU[e];
        }
      }
    }
  }
}

// :600-610: the (parallel, image) partials in order, divided by E keV
__global__ void general_reduce_kernel(GeneralArgs a) {
  const int n = a.N_E * a.N_P;
  const int ns = a.stokes ? 3 : 1;
  const int c = blockIdx.y;  // I, Q, U
  const int64_t n_ri = (int64_t)a.S0 * a.IOmax;
  double *out = c == 0 ? a.flux : (c == 1 ? a.flux_q : a.flux_u);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int64_t ri = 0; ri < n_ri; ri++) {
      const int row = (int)(ri / a.IOmax), I = (int)(ri - (int64_t)row * a.IOmax);
      if (I < a.n_img[row]) s += a.partial[(ri * ns + c) * n + t];
    }
    const int p = t / a.N_P;
    out[t] = s / (a.energies[p] * kKeV);
  }
}

}  // namespace

size_t general_geometry_smem_bytes(int N_R, int N_L) {
  return (size_t)(N_R + 8 * N_L + 12 * N_L + 7 * N_L) * sizeof(double) +
         (size_t)(4 * N_L + 4) * sizeof(int);
}

int launch_general(const GeneralArgs &a, cudaStream_t st) {
  if (a.S0 <= 0) return 0;
  const size_t smem = general_geometry_smem_bytes(a.N_R, a.N_L);
  const size_t smem_acc = (size_t)2 * a.S1 * sizeof(double);
  if (smem > 227 * 1024 || smem_acc > 227 * 1024) return -2;
  if (cudaFuncSetAttribute(general_geometry_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return -5;
  general_geometry_kernel<<<a.S0, kGenThreads, smem, st>>>(a);
  general_accumulate_kernel<<<(unsigned)((int64_t)a.S0 * a.IOmax), kGenAccThreads, smem_acc,
                              st>>>(a);
  const int n = a.N_E * a.N_P;
  general_reduce_kernel<<<dim3((n + 255) / 256, a.stokes ? 3 : 1), 256, 0, st>>>(a);
  return cudaGetLastError() == cudaSuccess ? 0 : -5;
}

}  // namespace xg
