// CPU oracle for the FDTD stepping path -- TEST INFRASTRUCTURE ONLY.
//
// A plain-loop restatement of the reference's per-point arithmetic, run on
// the host, behind the same Backend interface as the CUDA engine so that the
// C ABI (mfd.h) and the meep:: drop-in can be pointed at either.  Only the
// tests, __graft_entry__.smoke() and bench.py's cpu_baseline leg use it, as the
// checker / CPU baseline; the product library never links it.
//
// Each routine cites the reference code it restates:
//   curl (B, D)         step_curl                 src/step_generic.cpp:65-249
//   constitutive (E, H) step_update_EDHB          src/step_generic.cpp:566-785
//                       fields_chunk::update_eh   src/update_eh.cpp:66-213
//   polarisation        lorentzian::update_P      src/susceptibility.cpp:188-262
//                       subtract_P                src/susceptibility.cpp:264-281
//   sources             fields_chunk::step_source src/step.cpp:295-318
//   DFT                 dft_chunk::update_dft     src/dft.cpp:266-308
//   flux                dft_flux::flux            src/dft.cpp:542-556
//   scale_dft           dft_chunk::scale_dft      src/dft.cpp:402-406
//   far fields          dft_near2far::farfield_lowlevel src/near2far.cpp:334-378
//                       green3d / green2d         src/near2far.cpp:131-245
// The per-chunk choice of formula is made per point from its chunk region
// (Plan::region), see meep_gb300/csrc/mfd_plan.hpp.
#include "geom_eval.hpp"
#include "greens.hpp"
#include "subpixel.hpp"
#include <chrono>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "mfd_backend.hpp"

namespace mfd {
namespace {

static const double pi = 3.141592653589793238462643383276;

template <typename R> class CpuBackend : public Backend {
public:
  explicit CpuBackend(const Plan &) {}

  std::vector<R> f[NC], fu[NC], fw[NC], fcnd[NC], fmp[NC];
  std::vector<R> chi[NC], cnd[NC], cndinv[NC];
  std::vector<R> chioff[3][2]; // off-diagonal chi1inv of E along d, terms in Plan::offdiag order
  std::vector<R> sig[3], kap[3], siginv[3];
  struct PoleData {
    std::vector<R> P[3], PP[3], s[3];
    R gamma1inv, gamma1, omega0dtsqr, omega0dtsqr_denom;
  };
  std::vector<PoleData> poles;
  std::vector<std::vector<std::complex<double>>> dft;
  bool have_H_sep[NC] = {};
  double ms = 0;

  // complex (Bloch) fields: imaginary parts of every state array, swapped in
  // for the second pass of each half-step; `part` selects Re or Im of the
  // complex source amplitudes
  bool cplx = false;
  int part = 0;
  std::vector<R> f_im[NC], fu_im[NC], fw_im[NC], fcnd_im[NC], fmp_im[NC];
  std::vector<std::vector<R>> P_im, PP_im; // [pole * 3 + d]
  void swap_parts() {
    for (int c = 0; c < NC; c++) {
      f[c].swap(f_im[c]);
      fu[c].swap(fu_im[c]);
      fw[c].swap(fw_im[c]);
      fcnd[c].swap(fcnd_im[c]);
      fmp[c].swap(fmp_im[c]);
    }
    for (size_t q = 0; q < poles.size(); q++)
      for (int d = 0; d < 3; d++) {
        poles[q].P[d].swap(P_im[q * 3 + d]);
        poles[q].PP[d].swap(PP_im[q * 3 + d]);
      }
    part ^= 1;
  }
  double src_part(const std::complex<double> &A) const { return part ? A.imag() : A.real(); }

  // not-owned points of Bloch-periodic directions: position 0 of shift-0
  // components = conj(eikna) x position 2N, position 2N+1 of shift-1
  // components = eikna x position 1 (src/boundaries.cpp:207-229,
  // src/step.cpp:172-222); product in complex<realnum>
  // ghost plane along periodic d of one array (with its imaginary part for
  // complex fields) of a component whose shift along d is shift0 ? 0 : 1
  void ghost_plane(const Plan &p, int d, bool shift0, std::vector<R> &re, std::vector<R> *im) {
    int o1 = (d + 1) % 3, o2 = (d + 2) % 3;
    if (o1 > o2) std::swap(o1, o2);
    const std::complex<double> ph = shift0 ? std::conj(p.eikna[d]) : p.eikna[d];
    const std::complex<R> phr(R(ph.real()), R(ph.imag()));
    const int64_t dst = shift0 ? 0 : (int64_t)p.N[d] * p.stride[d];
    const int64_t src = shift0 ? (int64_t)p.N[d] * p.stride[d] : 0;
    for (int j1 = 0; j1 < p.ext[o1]; j1++)
      for (int j2 = 0; j2 < p.ext[o2]; j2++) {
        const int64_t o = j1 * p.stride[o1] + j2 * p.stride[o2];
        if (im) {
          const std::complex<R> v = phr * std::complex<R>(re[src + o], (*im)[src + o]);
          re[dst + o] = v.real();
          (*im)[dst + o] = v.imag();
        }
        else
          re[dst + o] = phr.real() * re[src + o];
      }
  }
  void ghost_copy(const Plan &p, int t0, int t1) {
    for (int d = 0; d < 3; d++) {
      if (!p.periodic[d]) continue;
      for (int c = 0; c < NC; c++) {
        if (f[c].empty() || (ctype(c) != t0 && ctype(c) != t1)) continue;
        ghost_plane(p, d, p.shift[c][d] == 0, f[c], cplx ? &f_im[c] : nullptr);
      }
    }
  }
  // polarizations of E at the not-owned points (the reference's PE_stuff
  // boundary step, src/step.cpp:116-119); read by the off-diagonal update
  void ghost_copy_pols(const Plan &p) {
    for (int d = 0; d < 3; d++) {
      if (!p.periodic[d]) continue;
      for (size_t q = 0; q < poles.size(); q++)
        for (int e = 0; e < 3; e++) {
          if (poles[q].P[e].empty()) continue;
          const bool s0 = p.shift[comp(MFD_E, e)][d] == 0;
          ghost_plane(p, d, s0, poles[q].P[e], cplx ? &P_im[q * 3 + e] : nullptr);
        }
    }
  }

  int64_t idx(const Plan &p, int k0, int k1, int k2) const {
    return k0 * p.stride[0] + k1 * p.stride[1] + k2 * p.stride[2];
  }

  std::vector<R> to_store(const Plan &p, const std::vector<double> &dense, double dflt) {
    std::vector<R> out(p.nstore, R(0));
    if (dense.empty()) {
      for (int64_t di = 0; di < p.ndense; di++)
        out[p.store_index_of_dense(di)] = R(dflt);
      return out;
    }
    for (int64_t di = 0; di < p.ndense; di++)
      out[p.store_index_of_dense(di)] = R(dense[di]);
    return out;
  }

  void setup(Plan &p) override {
    p.apply_matgrids_host();
    p.plan_offdiag();
    for (int c = 0; c < NC; c++) {
      if (!p.have[c]) continue;
      f[c].assign(p.nstore, R(0));
      int t = ctype(c), d = cdir(c);
      if (t == MFD_D || t == MFD_B) {
        fu[c].assign(p.nstore, R(0));
        fcnd[c].assign(p.nstore, R(0));
        if (!p.cond[c].empty()) {
          cnd[c] = to_store(p, p.cond[c], 0.0);
          cndinv[c].assign(p.nstore, R(1));
          // update_condinv (src/structure.cpp:693-707)
          for (int64_t i = 0; i < p.nstore; i++)
            cndinv[c][i] = R(1 / (1 + double(cnd[c][i]) * p.dt * 0.5));
        }
      }
      if (t == MFD_E || t == MFD_H) {
        fw[c].assign(p.nstore, R(0));
        if (t == MFD_E) {
          chi[c] = to_store(p, p.chi1inv[c][d], 1.0);
          for (int q = 0; q < p.offdiag[d].n; q++)
            chioff[d][q] = to_store(p, p.chi1inv[c][p.offdiag[d].dir[q]], 0.0);
          fmp[comp(MFD_D, d)].assign(p.nstore, R(0));
        }
        else {
          for (int dd = 0; dd < 3; dd++)
            if (!p.chi1inv[c][dd].empty()) {
              bool nontrivial = false;
              for (double v : p.chi1inv[c][dd])
                nontrivial = nontrivial || v != (dd == d ? 1.0 : 0.0);
              if (nontrivial) throw Error("mu != 1 is not supported");
            }
        }
      }
    }
    for (int d = 0; d < 3; d++) {
      sig[d].resize(p.sig[d].size());
      kap[d].resize(p.sig[d].size());
      siginv[d].resize(p.sig[d].size());
      for (size_t i = 0; i < p.sig[d].size(); i++) {
        sig[d][i] = R(p.sig[d][i]);
        kap[d][i] = R(p.kap[d][i]);
        // siginv from the stored (realnum) kap and sig, src/structure.cpp:687
        siginv[d][i] = p.sig[d][i] == 0.0 && p.kap[d][i] == 1.0 ? R(1) : R(1) / (kap[d][i] + sig[d][i]);
      }
    }
    // lorentzian coefficients (src/susceptibility.cpp:191-196)
    for (const Pole &pl : p.poles) {
      PoleData pd;
      R omega_0 = R(pl.omega0), gamma = R(pl.gamma), dt = R(p.dt);
      const R omega2pi = R(2 * pi * omega_0), g2pi = R(gamma * 2 * pi);
      pd.omega0dtsqr = omega2pi * omega2pi * dt * dt;
      pd.gamma1inv = R(1) / (R(1) + g2pi * dt / R(2));
      pd.gamma1 = (R(1) - g2pi * dt / R(2));
      pd.omega0dtsqr_denom = pl.drude ? R(0) : pd.omega0dtsqr;
      bool anyP = false;
      for (int d = 0; d < 3; d++) {
        int ec = comp(MFD_E, d);
        if (!p.have[ec] || pl.sigma[d].empty()) continue;
        pd.s[d] = to_store(p, pl.sigma[d], 0.0);
        pd.P[d].assign(p.nstore, R(0));
        pd.PP[d].assign(p.nstore, R(0));
        anyP = true;
      }
      (void)anyP;
      poles.push_back(std::move(pd));
    }
    cplx = p.complex_fields;
    if (cplx) {
      for (int c = 0; c < NC; c++) {
        f_im[c].assign(f[c].size(), R(0));
        fu_im[c].assign(fu[c].size(), R(0));
        fw_im[c].assign(fw[c].size(), R(0));
        fcnd_im[c].assign(fcnd[c].size(), R(0));
        fmp_im[c].assign(fmp[c].size(), R(0));
      }
      for (const PoleData &pd : poles)
        for (int d = 0; d < 3; d++) {
          P_im.emplace_back(pd.P[d].size(), R(0));
          PP_im.emplace_back(pd.PP[d].size(), R(0));
        }
    }
  }

  void add_monitor(Plan &p, int id) override {
    if ((int)dft.size() <= id) dft.resize(id + 1);
    const Monitor &m = p.monitors[id];
    dft[id].assign(m.npts * m.freq.size(), std::complex<double>(0, 0));
  }

  // ------------------------------------------------------------- curl
  void curl(Plan &p, int c) {
    const Plan::Curl &cp = p.curl[c];
    if (cp.g1 < 0) return;
    const int t = ctype(c);
    const R dtdx = cp.flip ? -R(p.g.courant) : R(p.g.courant);
    const R dt2 = R(p.dt) * R(0.5);
    R *F = f[c].data(), *FU = fu[c].data(), *FC = fcnd[c].data();
    const R *CND = cnd[c].empty() ? nullptr : cnd[c].data();
    const R *CNDINV = cndinv[c].empty() ? nullptr : cndinv[c].data();
    const int g1c = cp.g1, g2c = cp.g2;
    const int64_t s1 = cp.s1, s2 = cp.s2;
    const int dsig = cp.dsig, dsigu = cp.dsigu;
    const int *klo = p.klo[c], *khi = p.khi[c];
#pragma omp parallel for schedule(static)
    for (int k0 = klo[0]; k0 <= khi[0]; k0++)
      for (int k1 = klo[1]; k1 <= khi[1]; k1++)
        for (int k2 = klo[2]; k2 <= khi[2]; k2++) {
          const int k[3] = {k0, k1, k2};
          const int64_t i = idx(p, k0, k1, k2);
          // D curls read H where H is a separate array (PML slab along the H
          // component's own direction), B elsewhere (H == B aliasing,
          // src/fields.cpp:487-494, src/update_eh.cpp:163-171)
          const R *G1 = src_array(p, g1c, k);
          const R *G2 = g2c >= 0 ? src_array(p, g2c, k) : nullptr;
          R X = G1[i + s1] - G1[i];
          if (G2) X = X + G2[i] - G2[i + s2];
          bool sg = dsig >= 0 && p.in_slab(dsig, p.shift[c][dsig] + 2 * k[dsig]);
          bool su = dsigu >= 0 && p.in_slab(dsigu, p.shift[c][dsigu] + 2 * k[dsigu]);
          bool hc = CND != nullptr;
          if (sg && hc) {
            int r[3];
            for (int d = 0; d < 3; d++)
              r[d] = p.region(d, p.shift[c][d] + 2 * k[d]);
            hc = p.cond_chunk[c][r[0] * 9 + r[1] * 3 + r[2]] != 0;
          }
          if (!sg) {
            if (!su) {
              if (hc) F[i] = ((R(1) - dt2 * CND[i]) * F[i] - dtdx * X) * CNDINV[i];
              else F[i] -= dtdx * X;
            }
            else {
              const int ku = p.shift[c][dsigu] + 2 * k[dsigu];
              R fprev = FU[i];
              if (hc) FU[i] = ((R(1) - dt2 * CND[i]) * fprev - dtdx * X) * CNDINV[i];
              else FU[i] -= dtdx * X;
              F[i] = siginv[dsigu][ku] * ((kap[dsigu][ku] - sig[dsigu][ku]) * F[i] + FU[i] - fprev);
            }
          }
          else {
            const int kk = p.shift[c][dsig] + 2 * k[dsig];
            if (!su) {
              if (hc) {
                R fcp = FC[i];
                FC[i] = ((R(1) - dt2 * CND[i]) * FC[i] - dtdx * X) * CNDINV[i];
                F[i] = ((kap[dsig][kk] - sig[dsig][kk]) * F[i] + (FC[i] - fcp)) * siginv[dsig][kk];
              }
              else
                F[i] = ((kap[dsig][kk] - sig[dsig][kk]) * F[i] - dtdx * X) * siginv[dsig][kk];
            }
            else {
              const int ku = p.shift[c][dsigu] + 2 * k[dsigu];
              R fprev = FU[i];
              if (hc) {
                R fcp = FC[i];
                FC[i] = ((R(1) - dt2 * CND[i]) * FC[i] - dtdx * X) * CNDINV[i];
                FU[i] = ((kap[dsig][kk] - sig[dsig][kk]) * FU[i] + (FC[i] - fcp)) * siginv[dsig][kk];
              }
              else
                FU[i] = ((kap[dsig][kk] - sig[dsig][kk]) * FU[i] - dtdx * X) * siginv[dsig][kk];
              F[i] = siginv[dsigu][ku] * ((kap[dsigu][ku] - sig[dsigu][ku]) * F[i] + FU[i] - fprev);
            }
          }
        }
    (void)t;
  }

  // E/H component arrays as seen by a curl: H is separate from B only inside
  // the PML slab along the H component's own direction.
  const R *src_array(const Plan &p, int gc, const int k[3]) {
    if (ctype(gc) == MFD_H) {
      int d = cdir(gc);
      int bc = comp(MFD_B, d);
      if (p.pml_dir[d] && p.in_slab(d, p.shift[gc][d] + 2 * k[d])) return f[gc].data();
      return f[bc].data();
    }
    return f[gc].data();
  }

  // ------------------------------------------------------ H from B (PML)
  void update_h(Plan &p, int hc) {
    int d = cdir(hc), bc = comp(MFD_B, d);
    if (!p.pml_dir[d]) return;
    R *H = f[hc].data(), *FW = fw[hc].data();
    const R *Bf = f[bc].data();
    const int *klo = p.klo[hc], *khi = p.khi[hc];
#pragma omp parallel for schedule(static)
    for (int k0 = klo[0]; k0 <= khi[0]; k0++)
      for (int k1 = klo[1]; k1 <= khi[1]; k1++)
        for (int k2 = klo[2]; k2 <= khi[2]; k2++) {
          const int k[3] = {k0, k1, k2};
          const int kw = p.shift[hc][d] + 2 * k[d];
          if (!p.in_slab(d, kw)) continue;
          const int64_t i = idx(p, k0, k1, k2);
          R fwprev = FW[i], kapwkw = kap[d][kw], sigwkw = sig[d][kw];
          FW[i] = Bf[i];
          H[i] += (kapwkw + sigwkw) * FW[i] - (kapwkw - sigwkw) * fwprev;
        }
  }

  // -------------------------------------------- E from D - P, then pols
  void update_e(Plan &p, const std::vector<SrcStepValues> &vals) {
    // f_minus_p = D - P (list order) - integrated sources (src/update_eh.cpp:108-137)
    for (int d = 0; d < 3; d++) {
      int ec = comp(MFD_E, d), dc = comp(MFD_D, d);
      if (!p.have[ec]) continue;
      std::vector<R> &m = fmp[dc];
      std::memcpy(m.data(), f[dc].data(), sizeof(R) * p.nstore);
      for (PoleData &pd : poles)
        if (!pd.P[d].empty())
          for (int64_t i = 0; i < p.nstore; i++)
            m[i] -= pd.P[d][i];
    }
    for (const SourceGroup &sg : p.sources) {
      if (ctype(sg.c) != MFD_E || !p.srcs[sg.src].integrated) continue;
      int dc = comp(MFD_D, cdir(sg.c));
      for (size_t j = 0; j < sg.idx.size(); j++) {
        std::complex<double> A = sg.amp[j] * vals[sg.src].dip_e;
        fmp[dc][p.store_index_of_dense(sg.idx[j])] -= R(src_part(A));
      }
    }
    for (int d = 0; d < 3; d++) {
      int ec = comp(MFD_E, d), dc = comp(MFD_D, d);
      if (!p.have[ec]) continue;
      R *E = f[ec].data(), *FW = fw[ec].data();
      const R *G = fmp[dc].data(), *U = chi[ec].data();
      const bool pml = p.pml_dir[d];
      const int *klo = p.klo[ec], *khi = p.khi[ec];
      // OFFDIAG(u, g, sx) = 0.25 ((g[i] + g[i-sx]) u[i] + (g[i+s] + g[i+s-sx]) u[i+s])
      // with s the stride along d (src/step_generic.cpp:580-582)
      const int noff = p.offdiag[d].n;
      const R *OG[2] = {nullptr, nullptr}, *OU[2] = {nullptr, nullptr};
      int64_t osx[2] = {0, 0};
      for (int q = 0; q < noff; q++) {
        const int od = p.offdiag[d].dir[q];
        OG[q] = fmp[comp(MFD_D, od)].data();
        OU[q] = chioff[d][q].data();
        osx[q] = p.stride[od];
      }
      const int64_t s = p.stride[d];
#pragma omp parallel for schedule(static)
      for (int k0 = klo[0]; k0 <= khi[0]; k0++)
        for (int k1 = klo[1]; k1 <= khi[1]; k1++)
          for (int k2 = klo[2]; k2 <= khi[2]; k2++) {
            const int k[3] = {k0, k1, k2};
            const int64_t i = idx(p, k0, k1, k2);
            const int kw = p.shift[ec][d] + 2 * k[d];
            R gs = G[i], us = U[i];
            R val = (gs * us);
            for (int q = 0; q < noff; q++) {
              const R *g = OG[q], *u = OU[q];
              const int64_t sx = osx[q];
              val = val + R(0.25) * ((g[i] + g[i - sx]) * u[i] + (g[i + s] + g[(i + s) - sx]) * u[i + s]);
            }
            if (pml && p.in_slab(d, kw)) {
              R fwprev = FW[i], kapwkw = kap[d][kw], sigwkw = sig[d][kw];
              FW[i] = val;
              E[i] += (kapwkw + sigwkw) * FW[i] - (kapwkw - sigwkw) * fwprev;
            }
            else
              E[i] = val;
          }
    }
    // update_pols(E): W = f_w inside the PML slab of the component, E elsewhere
    for (PoleData &pd : poles)
      for (int d = 0; d < 3; d++) {
        if (pd.P[d].empty()) continue;
        int ec = comp(MFD_E, d);
        R *P = pd.P[d].data(), *PP = pd.PP[d].data();
        const R *S = pd.s[d].data();
        const R *E = f[ec].data(), *FW = fw[ec].data();
        const bool pml = p.pml_dir[d];
        const int *klo = p.klo[ec], *khi = p.khi[ec];
        const R g1inv = pd.gamma1inv, g1 = pd.gamma1, w0 = pd.omega0dtsqr,
                w0d = pd.omega0dtsqr_denom;
#pragma omp parallel for schedule(static)
        for (int k0 = klo[0]; k0 <= khi[0]; k0++)
          for (int k1 = klo[1]; k1 <= khi[1]; k1++)
            for (int k2 = klo[2]; k2 <= khi[2]; k2++) {
              const int k[3] = {k0, k1, k2};
              const int64_t i = idx(p, k0, k1, k2);
              const int kw = p.shift[ec][d] + 2 * k[d];
              const R *W = (pml && p.in_slab(d, kw)) ? FW : E;
              R pcur = P[i];
              P[i] = g1inv * (pcur * (R(2) - w0d) - g1 * PP[i] + w0 * (S[i] * W[i]));
              PP[i] = pcur;
            }
      }
  }

  // step_source for current (non-integrated) sources (src/step.cpp:295-318)
  void step_source(Plan &p, int ft, const std::vector<SrcStepValues> &vals) {
    for (const SourceGroup &sg : p.sources) {
      bool mag = ctype(sg.c) == MFD_H;
      if ((ft == MFD_B) != mag) continue;
      if (p.srcs[sg.src].integrated) continue;
      int c = comp(ft, cdir(sg.c));
      std::complex<double> cur = ft == MFD_B ? vals[sg.src].cur_b : vals[sg.src].cur_d;
      const R *ci = cndinv[c].empty() ? nullptr : cndinv[c].data();
      for (size_t j = 0; j < sg.idx.size(); j++) {
        int64_t i = p.store_index_of_dense(sg.idx[j]);
        std::complex<double> A = sg.amp[j] * cur * p.dt;
        if (ci) A = A * double(ci[i]);
        f[c][i] -= R(src_part(A));
      }
    }
  }

  // ------------------------------------------------------------------ DFT
  void update_dft(Plan &p, int id, double time) {
    const Monitor &m = p.monitors[id];
    int nf = (int)m.freq.size();
    std::vector<std::complex<double>> ph(nf);
    for (int w = 0; w < nf; w++)
      ph[w] = std::polar(1.0, 2 * pi * m.freq[w] * time) * m.scale;
    std::vector<std::complex<R>> phr(nf);
    for (int w = 0; w < nf; w++)
      phr[w] = std::complex<R>(R(ph[w].real()), R(ph[w].imag()));
    // centred-grid averaging directions (grid_volume::yee2cent_offsets,
    // src/vec.cpp:327-345): the first and second direction with shift 0
    int ad[2] = {-1, -1};
    if (m.centered)
      for (int d = 0; d < 3; d++)
        if (p.present[d] && p.shift[m.c][d] == 0) {
          if (ad[0] >= 0) ad[1] = d;
          else ad[0] = d;
        }
    int n[3];
    for (int d = 0; d < 3; d++)
      n[d] = m.hi[d] - m.lo[d] + 1;
    std::vector<std::complex<double>> &acc = dft[id];
    int64_t cnt = 0;
    for (int k0 = 0; k0 < n[0]; k0++)
      for (int k1 = 0; k1 < n[1]; k1++)
        for (int k2 = 0; k2 < n[2]; k2++, cnt++) {
          int kk[3] = {m.lo[0] + k0, m.lo[1] + k1, m.lo[2] + k2};
          // weight product in the reference's loop order: W3 * (W2 * (dV * W1)),
          // loop directions X,Y,Z in 3-D and Z(absent),X,Y in 2-D (IVEC_LOOP_WEIGHT)
          double wgt = 1.0;
          if (m.include_weights) {
            double wx = p.present[0] ? m.w[0][k0] : 1.0;
            double wy = p.present[1] ? m.w[1][k1] : 1.0;
            double wz = p.present[2] ? m.w[2][k2] : 1.0;
            if (p.g.dim == 2) wgt = wy * (wx * (m.dV * 1.0));
            else if (p.g.dim == 3) wgt = wz * (wy * (m.dV * wx));
            else wgt = 1.0 * (1.0 * (m.dV * wz));
            if (m.sqrt_weights) wgt = std::sqrt(wgt); // src/dft.cpp:279-280
          }
          R fv, fvi = R(0);
          if (cplx) {
            swap_parts();
            fvi = dft_value(p, m.c, kk, ad, wgt);
            swap_parts();
          }
          if (ad[1] >= 0) {
            int q1[3] = {kk[0], kk[1], kk[2]}, q2[3] = {kk[0], kk[1], kk[2]}, q3[3] = {kk[0], kk[1], kk[2]};
            q1[ad[0]]++;
            q2[ad[1]]++;
            q3[ad[0]]++;
            q3[ad[1]]++;
            fv = R((wgt * 0.25) * (value(p, m.c, kk) + value(p, m.c, q1) + value(p, m.c, q2) +
                                   value(p, m.c, q3)));
          }
          else if (ad[0] >= 0) {
            int q1[3] = {kk[0], kk[1], kk[2]};
            q1[ad[0]]++;
            fv = R((wgt * 0.5) * (value(p, m.c, kk) + value(p, m.c, q1)));
          }
          else
            fv = R(wgt * value(p, m.c, kk));
          if (cplx) {
            // dft += phase * complex(f_re, f_im) in complex<realnum> (src/dft.cpp:296-299)
            const std::complex<R> fc(fv, fvi);
            for (int w = 0; w < nf; w++) {
              const std::complex<R> q = phr[w] * fc;
              acc[cnt * nf + w] += std::complex<double>(double(q.real()), double(q.imag()));
            }
          }
          else
            for (int w = 0; w < nf; w++)
              acc[cnt * nf + w] += std::complex<double>(double(fv * phr[w].real()), double(fv * phr[w].imag()));
        }
  }

  // the (weighted, centred) monitor value at point kk
  R dft_value(const Plan &p, int c, const int kk[3], const int ad[2], double wgt) const {
    if (ad[1] >= 0) {
      int q1[3] = {kk[0], kk[1], kk[2]}, q2[3] = {kk[0], kk[1], kk[2]}, q3[3] = {kk[0], kk[1], kk[2]};
      q1[ad[0]]++;
      q2[ad[1]]++;
      q3[ad[0]]++;
      q3[ad[1]]++;
      return R((wgt * 0.25) * (value(p, c, kk) + value(p, c, q1) + value(p, c, q2) + value(p, c, q3)));
    }
    if (ad[0] >= 0) {
      int q1[3] = {kk[0], kk[1], kk[2]};
      q1[ad[0]]++;
      return R((wgt * 0.5) * (value(p, c, kk) + value(p, c, q1)));
    }
    return R(wgt * value(p, c, kk));
  }

  // value of component c at point k; H is read from B where the owning chunk
  // has no separate H array
  R value(const Plan &p, int c, const int k[3]) const {
    int64_t i = idx(p, k[0], k[1], k[2]);
    if (ctype(c) == MFD_H) {
      int d = cdir(c);
      if (!(p.pml_dir[d] && p.in_slab(d, p.shift[c][d] + 2 * k[d]))) return f[comp(MFD_B, d)][i];
    }
    return f[c][i];
  }

  void step(Plan &p, int64_t t, const std::vector<SrcStepValues> &vals) override {
    auto t0 = std::chrono::steady_clock::now();
    const int nparts = cplx ? 2 : 1;
    for (int q = 0; q < nparts; q++) {
      if (q) swap_parts();
      for (int d = 0; d < 3; d++)
        if (p.have[comp(MFD_B, d)]) curl(p, comp(MFD_B, d));
      step_source(p, MFD_B, vals);
      for (int d = 0; d < 3; d++)
        if (p.have[comp(MFD_H, d)]) update_h(p, comp(MFD_H, d));
      if (q) swap_parts();
    }
    ghost_copy(p, MFD_B, MFD_H);
    for (int q = 0; q < nparts; q++) {
      if (q) swap_parts();
      for (int d = 0; d < 3; d++)
        if (p.have[comp(MFD_D, d)]) curl(p, comp(MFD_D, d));
      step_source(p, MFD_D, vals);
      if (!p.any_offdiag) update_e(p, vals);
      if (q) swap_parts();
    }
    if (p.any_offdiag) {
      // the off-diagonal terms read D (and P) at the not-owned points: fill
      // them first, as the reference's D boundary step does before update_eh
      ghost_copy(p, MFD_D, MFD_D);
      for (int q = 0; q < nparts; q++) {
        if (q) swap_parts();
        update_e(p, vals);
        if (q) swap_parts();
      }
      ghost_copy_pols(p);
    }
    ghost_copy(p, MFD_D, MFD_E);
    int64_t tn = t + 1;
    for (size_t id = 0; id < p.monitors.size(); id++) {
      const Monitor &m = p.monitors[id];
      if (tn % m.decimation != 0) continue;
      double timeE = tn * p.dt;
      double time = ctype(m.c) == MFD_H || ctype(m.c) == MFD_B ? timeE - 0.5 * p.dt : timeE;
      update_dft(p, (int)id, time);
    }
    ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (!std::isfinite(center_energy(p))) throw Error("simulation fields are NaN or Inf");
  }

  // get_field(D_EnergyDensity, gv.center()) of fields::step()'s divergence
  // test (src/step.cpp:137-138): half the sum of Re(conj(E_d) D_d) with both
  // interpolated at the centre (Plan::center_probe)
  double center_energy(const Plan &p) const {
    double sum = 0.0;
    for (int d = 0; d < 3; d++) {
      const int ce = comp(MFD_E, d), cd = comp(MFD_D, d);
      if (!p.have[ce] || !p.have[cd]) continue;
      const Plan::ProbePoints pp = p.center_probe(d);
      double er = 0, dr = 0, ei = 0, dimg = 0;
      for (int j = 0; j < pp.n; j++) {
        er += pp.w[j] * double(f[ce][pp.idx[j]]);
        dr += pp.w[j] * double(f[cd][pp.idx[j]]);
        if (cplx) {
          ei += pp.w[j] * double(f_im[ce][pp.idx[j]]);
          dimg += pp.w[j] * double(f_im[cd][pp.idx[j]]);
        }
      }
      sum += er * dr + ei * dimg;
    }
    return sum * 0.5;
  }

  void begin_steps() override { ms = 0; }
  double last_step_ms() const override { return ms; }

  void get_field(Plan &p, int c, double *out) override {
    const std::vector<R> *src = &f[c];
    int t = ctype(c), d = cdir(c);
    for (int64_t di = 0; di < p.ndense; di++) {
      int k[3];
      p.dense_coords(di, k);
      int64_t i = idx(p, k[0], k[1], k[2]);
      const std::vector<R> *s = src;
      if (t == MFD_H && !(p.pml_dir[d] && p.in_slab(d, p.shift[c][d] + 2 * k[d])))
        s = &f[comp(MFD_B, d)];
      out[di] = double((*s)[i]);
    }
  }

  void get_field_im(Plan &p, int c, double *out) override {
    if (!cplx) {
      std::fill(out, out + p.ndense, 0.0);
      return;
    }
    swap_parts();
    get_field(p, c, out);
    swap_parts();
  }

  void get_dft(Plan &p, int id, double *out) override {
    const std::vector<std::complex<double>> &a = dft[id];
    for (size_t i = 0; i < a.size(); i++) {
      out[2 * i] = a[i].real();
      out[2 * i + 1] = a[i].imag();
    }
    (void)p;
  }

  void flux(Plan &p, int npairs, const int *idE, const int *idH, double *out) override {
    size_t nf = p.monitors[idE[0]].freq.size();
    for (size_t w = 0; w < nf; w++)
      out[w] = 0;
    for (int q = 0; q < npairs; q++) {
      const auto &E = dft[idE[q]], &H = dft[idH[q]];
      size_t np = p.monitors[idE[q]].npts;
      for (size_t k = 0; k < np; k++)
        for (size_t w = 0; w < nf; w++)
          out[w] += real(E[k * nf + w] * conj(H[k * nf + w]));
    }
  }

  void set_dft(Plan &p, int id, const double *in) override {
    std::vector<std::complex<double>> &a = dft[id];
    for (size_t i = 0; i < a.size(); i++)
      a[i] = std::complex<double>(in[2 * i], in[2 * i + 1]);
    (void)p;
  }

  void scale_dft(Plan &p, int id, std::complex<double> s) override {
    for (auto &v : dft[id]) v *= s;
    (void)p;
  }

  // the reference's loop: per far point, sheets in list order, then per
  // frequency the sheet's points in order and their periodic images
  void farfield(Plan &p, const N2FSpec &s, const std::vector<N2FSheet> &sheets, int64_t nx, const double *x,
                double *out) override {
    using mgb_green::cplx;
    const size_t nf = p.monitors[sheets[0].id].freq.size();
    const std::vector<double> &freq = p.monitors[sheets[0].id].freq;
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t ix = 0; ix < nx; ix++) {
      std::vector<std::complex<double>> EH(6 * nf, 0.0);
      const double xf[3] = {x[3 * ix], x[3 * ix + 1], s.dim == 2 ? 0.0 : x[3 * ix + 2]};
      for (const N2FSheet &sh : sheets) {
        const Monitor &m = p.monitors[sh.id];
        const std::vector<std::complex<double>> &a = dft[sh.id];
        int n[3];
        for (int d = 0; d < 3; d++)
          n[d] = m.hi[d] - m.lo[d] + 1;
        for (size_t i = 0; i < nf; ++i) {
          size_t idx = 0;
          for (int k0 = 0; k0 < n[0]; k0++)
            for (int k1 = 0; k1 < n[1]; k1++)
              for (int k2 = 0; k2 < n[2]; k2++, idx++) {
                const int k[3] = {k0, k1, k2};
                double x0[3];
                for (int d = 0; d < 3; d++)
                  x0[d] = (sh.is_half[d] + k[d]) * s.inva + sh.rshift[d];
                if (s.dim == 2) x0[2] = 0.0;
                const std::complex<double> J = a[nf * idx + i];
                double xs[3] = {x0[0], x0[1], x0[2]};
                for (int i0 = -s.pn[0]; i0 <= s.pn[0]; ++i0) {
                  if (s.pdir[0] >= 0) xs[s.pdir[0]] = x0[s.pdir[0]] + i0 * s.period[0];
                  const double phase0 = i0 * s.pk[0];
                  for (int i1 = -s.pn[1]; i1 <= s.pn[1]; ++i1) {
                    if (s.pdir[1] >= 0) xs[s.pdir[1]] = x0[s.pdir[1]] + i1 * s.period[1];
                    const double phase = phase0 + i1 * s.pk[1];
                    const std::complex<double> cphase = std::polar(1.0, phase);
                    cplx E6[6];
                    if (s.dim == 2) mgb_green::green2d(E6, xf, freq[i], s.eps, s.mu, xs, sh.c0, {J.real(), J.imag()});
                    else mgb_green::green3d(E6, xf, freq[i], s.eps, s.mu, xs, sh.c0, {J.real(), J.imag()});
                    for (int j = 0; j < 6; ++j)
                      EH[i * 6 + j] += std::complex<double>(E6[j].re, E6[j].im) * cphase;
                  }
                }
              }
        }
      }
      for (size_t q = 0; q < 6 * nf; q++) {
        out[(ix * 6 * nf + q) * 2] = EH[q].real();
        out[(ix * 6 * nf + q) * 2 + 1] = EH[q].imag();
      }
    }
  }
};

} // namespace

Backend *make_backend(const Plan &p) {
  if (p.g.precision == 64) return new CpuBackend<double>(p);
  return new CpuBackend<float>(p);
}

// mfd_subpixel_rows on the host: the shared averaging routine over the same
// object list, pixel by pixel (the reference's order of work)
void subpixel_rows(int dim, int cdir, int64_t npix, const double *lo, const double *hi, double tol, int maxeval,
                   int nobj, const mfd_object *objs, double eps_default, double *rows) {
  const mgb_subpixel::SphereQuad &sq = mgb_subpixel::sphere_quadrature();
  auto chi = [objs, nobj, eps_default](const double p[3]) {
    const int q = mgb_geom::object_at(objs, nobj, p);
    return q < 0 ? eps_default : objs[q].eps;
  };
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < npix; i++)
    mgb_subpixel::eff_chi1inv_row(dim, cdir, lo + 3 * i, hi + 3 * i, tol, maxeval, sq, chi, rows + 3 * i);
}

// mfd_green on the host
void green_eval(int dim, int c0, double freq, double eps, double mu, double f0re, double f0im, int64_t n,
                const double *x, const double *x0, double *out) {
  for (int64_t i = 0; i < n; i++) {
    mgb_green::cplx EH[6];
    if (dim == 2) mgb_green::green2d(EH, x + 3 * i, freq, eps, mu, x0 + 3 * i, c0, {f0re, f0im});
    else mgb_green::green3d(EH, x + 3 * i, freq, eps, mu, x0 + 3 * i, c0, {f0re, f0im});
    for (int c = 0; c < 6; c++) {
      out[12 * i + 2 * c] = EH[c].re;
      out[12 * i + 2 * c + 1] = EH[c].im;
    }
  }
}

} // namespace mfd
