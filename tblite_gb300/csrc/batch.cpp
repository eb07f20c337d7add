// Batched ensemble driver: GFN2-xTB / GFN1-xTB energy + gradient of many independent molecules with one
// launch per SCF step for a whole size bucket, instead of one launch per molecule.
//
// Layout.  Molecules are sorted by orbital count (largest first) and grouped into size buckets
// whose largest member sets the launch shape.  Every per-molecule array lives in one device
// arena, in three regions:
//   zeroed   S, H, D, Q and accumulators; then the results, zeroed and read back (one D2H)
//   scratch  matrices and vectors that the SCF writes before it reads them
//   uploaded basis, parameters, geometry and the start charges (one H2D from a pinned stage)
// MolPtrs (one per molecule, in device memory) holds the slice pointers; batched kernels walk a
// list of molecule indices with blockIdx.z and run the one-molecule arithmetic.
//
// SCF.  All molecules iterate in lockstep (the same iteration index, so the Broyden history
// index is shared); after each iteration one small D2H of the per-molecule flags drops the
// converged molecules from the launch lists.  The convergence test, the Broyden update and the
// Fermi filling run per molecule on the device with each molecule's own settings.
//
// A molecule leaves the batch for the one-molecule path (which then reproduces exactly what a
// plain call does, including its errors) when it is larger than the batched
// tridiagonalisation holds, uses temperature annealing, carries an implicit solvation model,
// would need more Broyden history than the batch keeps, has a
// Fermi level within 51 kT of the highest eigenvalue the SCF computes, does not converge within
// its iteration limit, or fails (overlap not positive definite, singular Broyden system).
// Molecules that ask for the parameter gradient get it in the batch, after the nuclear gradient.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <exception>
#include <mutex>
#include <numeric>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/tblite_gb300_ext.h"
#include "api_internal.h"

using namespace tb;

namespace tb {
int batch_tridiag_max_n();
}

namespace {

constexpr int HCAP = 48;  // Broyden history kept per molecule in the batch

struct Arena {
  char* dev = nullptr;
  size_t dev_cap = 0;
  char* host = nullptr;  // pinned stage for uploads and read-back
  size_t host_cap = 0;
  cudaStream_t stream = nullptr;
  // size buckets run concurrently on side streams, forked from and joined into `stream`
  static constexpr int NSIDE = 16;
  cudaStream_t side[NSIDE] = {};
  cudaEvent_t fork = nullptr, join[NSIDE] = {};
  void reserve(size_t dbytes, size_t hbytes) {
    if (dbytes > dev_cap) {
      if (dev) cudaFree(dev);
      dev = nullptr;
      cuda_check(cudaMalloc(&dev, dbytes), "batch arena");
      dev_cap = dbytes;
    }
    if (hbytes > host_cap) {
      if (host) cudaFreeHost(host);
      host = nullptr;
      cuda_check(cudaMallocHost(&host, hbytes), "batch stage");
      host_cap = hbytes;
    }
    if (!stream) {
      cuda_check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "stream");
      cuda_check(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming), "event");
      for (int k = 0; k < NSIDE; ++k) {
        cuda_check(cudaStreamCreateWithFlags(&side[k], cudaStreamNonBlocking), "stream");
        cuda_check(cudaEventCreateWithFlags(&join[k], cudaEventDisableTiming), "event");
      }
    }
  }
};
std::mutex g_batch_mutex;
Arena g_arena;
int g_last_fallbacks = 0;
// two calculators run in one chunk only with the same global model constants
static bool same_model(const ModelConstants& a, const ModelConstants& b) {
  if (a.pair_mode != b.pair_mode) return false;
  const double va[] = {a.wexp, a.enscale, a.kpol, a.gexp, a.rep_kexp, a.rep_klight, a.dmp3,
                       a.dmp5, a.mp_kexp, a.mp_shift, a.mp_rmax, a.s6, a.s8, a.a1, a.a2, a.s9};
  const double vb[] = {b.wexp, b.enscale, b.kpol, b.gexp, b.rep_kexp, b.rep_klight, b.dmp3,
                       b.dmp5, b.mp_kexp, b.mp_shift, b.mp_rmax, b.s6, b.s8, b.a1, b.a2, b.s9};
  for (size_t k = 0; k < sizeof(va) / sizeof(va[0]); ++k)
    if (!(va[k] == vb[k])) return false;
  for (int l = 0; l < 5; ++l)
    for (int m = 0; m < 5; ++m)
      if (!(a.ksh[l][m] == b.ksh[l][m])) return false;
  return true;
}

int g_batch_streams = 8;  // side streams the size buckets are spread over
bool g_batch_sp2 = true;  // closed shells of >= g_sp2_min_nao orbitals: density by projection
// schedule of the batch (set by hand or by tblite_gb300_batch_autotune): smallest orbital count
// of the projection, and the bucket cut (a bucket ends below cut_num/cut_den of its largest)
int g_sp2_min_nao = SP2_MIN_NAO;
int g_cut_num = 3, g_cut_den = 4;
std::string g_schedule_note = "defaults";
int g_last_projected = 0;  // molecules of the last call whose SCF density came from projection
bool g_batch_graphs = true;  // SCF iterations as CUDA graphs
int g_last_graph_builds = 0, g_last_graph_launches = 0;  // of the last call
double g_last_device_ms = 0.0;  // device time of the last call's batched steps (CUDA events)
// host wall time of the last call by phase (ms): plans, chunking, staging and upload, result
// unpacking, one-molecule path, whole call
enum { HP_PLAN, HP_CHUNK, HP_STAGE, HP_UNPACK, HP_PLAIN, HP_TOTAL, HP_N };
double g_last_host_ms[HP_N] = {};
using host_clock = std::chrono::steady_clock;
double ms_since(host_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(host_clock::now() - t0).count();
}

// fn(i) for i in [0, n) on up to 16 host threads in contiguous ranges (one thread below 256
// molecules); fn touches only molecule i's host data.  The first exception is rethrown.
template <class F>
void host_parallel(int n, F&& fn) {
  const int hw = std::max(1u, std::thread::hardware_concurrency());
  const int nt = std::max(1, std::min({hw, 16, n / 128}));
  if (nt == 1) {
    for (int i = 0; i < n; ++i) fn(i);
    return;
  }
  std::vector<std::exception_ptr> err(nt);
  auto work = [&](int t) {
    try {
      for (int i = (int)((long)n * t / nt), e = (int)((long)n * (t + 1) / nt); i < e; ++i) fn(i);
    } catch (...) {
      err[t] = std::current_exception();
    }
  };
  std::vector<std::thread> pool;
  pool.reserve(nt - 1);
  for (int t = 1; t < nt; ++t) pool.emplace_back(work, t);
  work(0);
  for (auto& th : pool) th.join();
  for (auto& e : err)
    if (e) std::rethrow_exception(e);
}
std::vector<int> g_last_iters;  // SCF iterations per molecule of the last call (0: not batched)
std::vector<int> g_last_modes;  // 1 projection, 0 diagonalisation, -1 one-molecule path

// byte offsets of one region, 256-byte aligned pieces
struct Region {
  size_t size = 0;
  size_t take(size_t bytes) {
    const size_t o = size;
    size += (bytes + 255) & ~(size_t)255;
    return o;
  }
};

enum { RZ = 0, RR = 1, RS = 2, RU = 3, NREG = 4 };  // zeroed, zeroed + read back, scratch, uploaded

struct Piece {  // where a field of a molecule lives
  int region;
  size_t off, bytes;
};

struct Plan {
  int idx;  // position in the caller's arrays
  _tblite_calculator* c;
  const _tblite_structure* mol;
  _tblite_result* res;
  int nat, nsh, nao, nd, memory, max_iter, method;
  int model = 0;  // index of the calculator's global model constants among the call's
  double nalp, nbet;
  bool has_d4, has_d3;
  bool param_grad;  // dE/d(shell parameters) with the single point
  int wbo_ch;       // bond-order channels: 0 not requested, 1 closed shell, 2 open shell
  bool molmom;      // molecular moments requested
  bool sp2;         // density by spectral projection during the SCF (sp2.cu)
  // offsets (region, offset) of every array
  Piece xyz, at_z, at_sh, sh_atom, sh_l, sh_nprim, sh_alpha, sh_coeff, sh_ao, ao_sh, ao_at, sh_se0,
      sh_kcn, sh_shpoly, sh_zeta, sh_hub, sh_gam3, sh_refocc, at_en, at_rad, at_rcov, at_mprad,
      at_vcn, at_dkern, at_qkern, at_repa, at_repz, sh_valence, at_gam3;
  Piece d3_sp, d3_nref, d3_refcn, d3_c6ref, d3_r4r2, d3_rcov, d3_cn, d3_w, d3_dw, d3_dEdcn;
  Piece d4_sp, d4_nref, d4_ngw, d4_refcn, d4_refq, d4_zeff, d4_gam, d4_r4r2, d4_rcov, d4_en,
      d4_c6ref;
  Piece d4_cn, d4_gw, d4_dgw, d4_gwv, d4_dgwdq, d4_dgwv_cn, d4_c6, d4_dc6, d4_e3, d4_dEdcn, d4_atm,
      d4_de;
  Piece cn, se, mrad, dmrdcn, ctab, S, H, D, Q, F, P, C, scratch, emo, focc;
  Piece qsh, qat, dpat, qpat, qsh_o, qat_o, dpat_o, qpat_o, vsh, vat, vdp, vqp, vao;
  Piece mull, eband, eelec, erep, vec_out, scal, icount;
  Piece bq, bqlast, bdq, bdqlast, bdf, bu, ba, bomega, bwork, bstatus;
  Piece grad, sigma, sig_at, dEdcn;
  Piece X, A, T1, Y, lu, ed, ee, etau, epv, escal, estatus, conv;
  Piece pgrad, zgrad;  // [4][nsh], [nsh] (param_grad only)
  Piece wbo;           // [wbo_ch][nat][nat] (bond orders requested only)
  Piece img, iexp, img2, iexp2, sp2s, sp2i, sp2p;  // spectral projection (sp2 only)
  Piece ximg0, ximg1, xexp0, xexp1;                 // X's slice images (sp2 only)
};

struct Bucket {
  int first, last;  // range in the sorted plan
  int nat_max = 0, nsh_max = 0, nao_max = 0, nd_max = 0;
  bool sp2 = false;
  int sp2_steps = SP2_MAX_STEPS;  // step budget of the next projection
};

template <class T>
Piece piece(Region* regs, int r, size_t count) {
  Piece p;
  p.region = r;
  p.bytes = sizeof(T) * std::max<size_t>(count, 1);
  p.off = regs[r].take(p.bytes);
  return p;
}

void layout(Plan& pl, Region* R) {
  const size_t na = pl.nat, ns = pl.nsh, n = pl.nao, nn = n * n, nd = pl.nd;
  const size_t hm = (size_t)std::min(pl.memory, HCAP);
  // uploaded: basis, parameters, geometry, start charges
  pl.xyz = piece<double>(R, RU, 3 * na);
  pl.at_z = piece<int>(R, RU, na);
  pl.at_sh = piece<int>(R, RU, na + 1);
  pl.sh_atom = piece<int>(R, RU, ns);
  pl.sh_l = piece<int>(R, RU, ns);
  pl.sh_nprim = piece<int>(R, RU, ns);
  pl.sh_alpha = piece<double>(R, RU, ns * MAXG);
  pl.sh_coeff = piece<double>(R, RU, ns * MAXG);
  pl.sh_ao = piece<int>(R, RU, ns);
  pl.ao_sh = piece<int>(R, RU, n);
  pl.ao_at = piece<int>(R, RU, n);
  for (Piece* p : {&pl.sh_se0, &pl.sh_kcn, &pl.sh_shpoly, &pl.sh_zeta, &pl.sh_hub, &pl.sh_gam3,
                   &pl.sh_refocc})
    *p = piece<double>(R, RU, ns);
  for (Piece* p : {&pl.at_en, &pl.at_rad, &pl.at_rcov, &pl.at_mprad, &pl.at_vcn, &pl.at_dkern,
                   &pl.at_qkern, &pl.at_repa, &pl.at_repz, &pl.at_gam3})
    *p = piece<double>(R, RU, na);
  pl.sh_valence = piece<int>(R, RU, ns);
  if (pl.has_d3) {
    pl.d3_nref = piece<int>(R, RU, na);
    pl.d3_refcn = piece<double>(R, RU, na * D4_MREF);
    pl.d3_sp = piece<int>(R, RU, na);
    pl.d3_c6ref = piece<double>(R, RU, pl.c->d3_c6ref.size());
    pl.d3_r4r2 = piece<double>(R, RU, na);
    pl.d3_rcov = piece<double>(R, RU, na);
    for (Piece* p : {&pl.d3_cn, &pl.d3_dEdcn}) *p = piece<double>(R, RS, na);
    for (Piece* p : {&pl.d3_w, &pl.d3_dw}) *p = piece<double>(R, RS, na * D4_MREF);
  }
  if (pl.has_d4) {
    pl.d4_sp = piece<int>(R, RU, na);
    pl.d4_nref = piece<int>(R, RU, na);
    pl.d4_ngw = piece<int>(R, RU, na * D4_MREF);
    pl.d4_refcn = piece<double>(R, RU, na * D4_MREF);
    pl.d4_refq = piece<double>(R, RU, na * D4_MREF);
    for (Piece* p : {&pl.d4_zeff, &pl.d4_gam, &pl.d4_r4r2, &pl.d4_rcov, &pl.d4_en})
      *p = piece<double>(R, RU, na);
    pl.d4_c6ref = piece<double>(R, RU, pl.c->d4_c6ref.size());
  }
  pl.qsh = piece<double>(R, RU, ns);
  pl.qat = piece<double>(R, RU, na);
  pl.dpat = piece<double>(R, RU, 3 * na);
  pl.qpat = piece<double>(R, RU, 6 * na);
  // zeroed: integrals (screened pairs stay zero), accumulators, results
  pl.S = piece<double>(R, RZ, nn);
  pl.H = piece<double>(R, RZ, nn);
  pl.D = piece<double>(R, RZ, 3 * nn);
  pl.Q = piece<double>(R, RZ, 6 * nn);
  pl.dEdcn = piece<double>(R, RZ, na);
  pl.conv = piece<double>(R, RZ, 3);
  pl.bstatus = piece<int>(R, RZ, 1);
  pl.estatus = piece<int>(R, RZ, 1);
  if (pl.has_d4) pl.d4_dEdcn = piece<double>(R, RZ, na);
  // zeroed and read back
  pl.grad = piece<double>(R, RR, 3 * na);
  pl.sig_at = piece<double>(R, RR, 9 * na);
  pl.sigma = piece<double>(R, RR, 9);
  pl.qsh_o = piece<double>(R, RR, ns);
  pl.qat_o = piece<double>(R, RR, na);
  pl.dpat_o = piece<double>(R, RR, 3 * na);
  pl.qpat_o = piece<double>(R, RR, 6 * na);
  pl.emo = piece<double>(R, RR, n);
  pl.focc = piece<double>(R, RR, 3 * n);
  pl.eelec = piece<double>(R, RR, na);
  pl.erep = piece<double>(R, RR, na);
  if (pl.has_d4) pl.d4_e3 = piece<double>(R, RR, na);
  if (pl.param_grad) {
    pl.pgrad = piece<double>(R, RR, 4 * ns);
    pl.zgrad = piece<double>(R, RR, ns);
  }
  if (pl.wbo_ch > 0) pl.wbo = piece<double>(R, RR, (size_t)pl.wbo_ch * na * na);
  if (pl.sp2) {
    pl.img = piece<uint16_t>(R, RS, pimage_bytes((int)n, (int)n) / sizeof(uint16_t));
    pl.iexp = piece<int>(R, RS, pimage_lines((int)n));
    pl.img2 = piece<uint16_t>(R, RS, pimage_bytes((int)n, (int)n) / sizeof(uint16_t));
    pl.iexp2 = piece<int>(R, RS, pimage_lines((int)n));
    pl.sp2s = piece<double>(R, RS, 8);
    pl.sp2i = piece<int>(R, RZ, 8);  // zeroed: the pipeline status starts clear
    pl.sp2p = piece<unsigned long long>(R, RS, 3 * (size_t)sp2_slot_count((int)n));
    pl.ximg0 = piece<uint16_t>(R, RS, pimage_bytes((int)n, (int)n) / sizeof(uint16_t));
    pl.ximg1 = piece<uint16_t>(R, RS, pimage_bytes((int)n, (int)n) / sizeof(uint16_t));
    pl.xexp0 = piece<int>(R, RS, pimage_lines((int)n));
    pl.xexp1 = piece<int>(R, RS, pimage_lines((int)n));
  }
  // scratch
  pl.cn = piece<double>(R, RS, na);
  pl.se = piece<double>(R, RS, ns);
  pl.mrad = piece<double>(R, RS, na);
  pl.ctab = piece<double>(R, RS, ns * ns + 3 * na * na);
  pl.dmrdcn = piece<double>(R, RS, na);
  for (Piece* p : {&pl.F, &pl.P, &pl.C, &pl.scratch, &pl.X, &pl.A, &pl.T1, &pl.Y})
    *p = piece<double>(R, RS, nn);
  pl.lu = piece<double>(R, RS, 5 * nn);
  pl.vsh = piece<double>(R, RS, ns);
  pl.vat = piece<double>(R, RS, na);
  pl.vdp = piece<double>(R, RS, 3 * na);
  pl.vqp = piece<double>(R, RS, 6 * na);
  pl.vao = piece<double>(R, RS, n);
  pl.mull = piece<double>(R, RS, (size_t)mulliken_chunks((int)n) * 11 * n);
  pl.eband = piece<double>(R, RS, na);
  pl.vec_out = piece<double>(R, RS, std::max(nd, n));
  pl.scal = piece<double>(R, RS, 8);
  pl.icount = piece<int>(R, RS, 4);
  for (Piece* p : {&pl.bq, &pl.bqlast, &pl.bdq, &pl.bdqlast}) *p = piece<double>(R, RS, nd);
  pl.bdf = piece<double>(R, RS, nd * hm);
  pl.bu = piece<double>(R, RS, nd * hm);
  pl.ba = piece<double>(R, RS, hm * hm);
  pl.bomega = piece<double>(R, RS, hm);
  pl.bwork = piece<double>(R, RS, hm * hm + 2 * hm + 64);
  pl.ed = piece<double>(R, RS, n + 1);
  pl.ee = piece<double>(R, RS, n + 1);
  pl.etau = piece<double>(R, RS, n + 1);
  pl.epv = piece<double>(R, RS, 4 * (n + 1));
  pl.escal = piece<double>(R, RS, 8);
  if (pl.has_d4) {
    pl.d4_cn = piece<double>(R, RS, na);
    for (Piece* p : {&pl.d4_gw, &pl.d4_dgw, &pl.d4_gwv, &pl.d4_dgwdq, &pl.d4_dgwv_cn})
      *p = piece<double>(R, RS, na * D4_MREF);
    pl.d4_c6 = piece<double>(R, RS, na * na);
    pl.d4_dc6 = piece<double>(R, RS, na * na);
    pl.d4_atm = piece<double>(R, RS, 8 * na * na);
    pl.d4_de = piece<double>(R, RS, na * na);
  }
}

struct Bases {
  char* base[NREG];
  template <class T>
  T* at(const Piece& p) const {
    return reinterpret_cast<T*>(base[p.region] + p.off);
  }
};

template <class T>
void stage(const Bases& hb, const Piece& p, const std::vector<T>& v) {
  if (!v.empty()) std::memcpy(hb.at<T>(p), v.data(), sizeof(T) * v.size());
}

MolPtrs make_ptrs(const Plan& pl, const Bases& db) {
  MolPtrs q{};
  DevMol& m = q.m;
  m.nat = pl.nat;
  m.nsh = pl.nsh;
  m.nao = pl.nao;
  m.xyz = db.at<double>(pl.xyz);
  m.at_z = db.at<int>(pl.at_z);
  m.at_sh = db.at<int>(pl.at_sh);
  m.sh_atom = db.at<int>(pl.sh_atom);
  m.sh_l = db.at<int>(pl.sh_l);
  m.sh_nprim = db.at<int>(pl.sh_nprim);
  m.sh_alpha = db.at<double>(pl.sh_alpha);
  m.sh_coeff = db.at<double>(pl.sh_coeff);
  m.sh_ao = db.at<int>(pl.sh_ao);
  m.ao_sh = db.at<int>(pl.ao_sh);
  m.ao_at = db.at<int>(pl.ao_at);
  m.sh_se0 = db.at<double>(pl.sh_se0);
  m.sh_kcn = db.at<double>(pl.sh_kcn);
  m.sh_shpoly = db.at<double>(pl.sh_shpoly);
  m.sh_zeta = db.at<double>(pl.sh_zeta);
  m.sh_hub = db.at<double>(pl.sh_hub);
  m.sh_gam3 = db.at<double>(pl.sh_gam3);
  m.sh_refocc = db.at<double>(pl.sh_refocc);
  m.at_en = db.at<double>(pl.at_en);
  m.at_rad = db.at<double>(pl.at_rad);
  m.at_rcov = db.at<double>(pl.at_rcov);
  m.at_mprad = db.at<double>(pl.at_mprad);
  m.at_vcn = db.at<double>(pl.at_vcn);
  m.at_dkern = db.at<double>(pl.at_dkern);
  m.at_qkern = db.at<double>(pl.at_qkern);
  m.at_repa = db.at<double>(pl.at_repa);
  m.at_repz = db.at<double>(pl.at_repz);
  m.sh_valence = db.at<int>(pl.sh_valence);
  m.at_gam3 = db.at<double>(pl.at_gam3);
  q.has_d4 = pl.has_d4 ? 1 : 0;
  q.has_d3 = pl.has_d3 ? 1 : 0;
  if (pl.has_d3) {
    DevD3& d = q.d3;
    d3_model_constants(d, pl.c);
    d.nsp = pl.c->d3_nsp;
    d.sp = db.at<int>(pl.d3_sp);
    d.nref = db.at<int>(pl.d3_nref);
    d.refcn = db.at<double>(pl.d3_refcn);
    d.c6ref = db.at<double>(pl.d3_c6ref);
    d.r4r2 = db.at<double>(pl.d3_r4r2);
    d.rcov = db.at<double>(pl.d3_rcov);
    d.cn = db.at<double>(pl.d3_cn);
    d.w = db.at<double>(pl.d3_w);
    d.dw = db.at<double>(pl.d3_dw);
    d.dEdcn = db.at<double>(pl.d3_dEdcn);
  }
  if (pl.has_d4) {
    DevD4& d = q.d4;
    d.nsp = pl.c->d4_nsp;
    d.sp = db.at<int>(pl.d4_sp);
    d.nref = db.at<int>(pl.d4_nref);
    d.ngw = db.at<int>(pl.d4_ngw);
    d.refcn = db.at<double>(pl.d4_refcn);
    d.refq = db.at<double>(pl.d4_refq);
    d.zeff = db.at<double>(pl.d4_zeff);
    d.gam = db.at<double>(pl.d4_gam);
    d.r4r2 = db.at<double>(pl.d4_r4r2);
    d.rcov = db.at<double>(pl.d4_rcov);
    d.en = db.at<double>(pl.d4_en);
    d.c6ref = db.at<double>(pl.d4_c6ref);
    d4_model_constants(d, pl.c);
    D4Work& w = q.d4w;
    w.cn = db.at<double>(pl.d4_cn);
    w.gw = db.at<double>(pl.d4_gw);
    w.dgw = db.at<double>(pl.d4_dgw);
    w.gwv = db.at<double>(pl.d4_gwv);
    w.dgwdq = db.at<double>(pl.d4_dgwdq);
    w.dgwv_cn = db.at<double>(pl.d4_dgwv_cn);
    w.c6 = db.at<double>(pl.d4_c6);
    w.dc6 = db.at<double>(pl.d4_dc6);
    w.e3 = db.at<double>(pl.d4_e3);
    w.dEdcn = db.at<double>(pl.d4_dEdcn);
    w.atm = db.at<double>(pl.d4_atm);
    w.de = db.at<double>(pl.d4_de);
  }
  q.nd = pl.nd;
  // GFN2-xTB mixes the atomic multipoles with the shell charges, GFN1-xTB the charges alone
  q.with_mp = pl.method == 2 ? 1 : 0;
  q.mull_chunks = mulliken_chunks(pl.nao);
  q.memory = std::min(pl.memory, HCAP);
  q.nev = scf_eigenvalue_count(pl.nao, std::max(pl.nalp, pl.nbet));
  q.nalp = pl.nalp;
  q.nbet = pl.nbet;
  q.kt = pl.c->etemp;
  q.damp = pl.c->damping;
  q.econv = 1.0e-6 * pl.c->accuracy;
  q.pconv = 2.0e-5 * pl.c->accuracy;
  q.h0_cutoff = gfn2_scalars(pl.c).h0_cutoff;
  q.cn = db.at<double>(pl.cn);
  q.se = db.at<double>(pl.se);
  q.mrad = db.at<double>(pl.mrad);
  q.ctab = db.at<double>(pl.ctab);
  q.dmrdcn = db.at<double>(pl.dmrdcn);
  q.S = db.at<double>(pl.S);
  q.H = db.at<double>(pl.H);
  q.D = db.at<double>(pl.D);
  q.Q = db.at<double>(pl.Q);
  q.F = db.at<double>(pl.F);
  q.P = db.at<double>(pl.P);
  q.C = db.at<double>(pl.C);
  q.scratch = db.at<double>(pl.scratch);
  q.emo = db.at<double>(pl.emo);
  q.focc = db.at<double>(pl.focc);
  q.qsh = db.at<double>(pl.qsh);
  q.qat = db.at<double>(pl.qat);
  q.dpat = db.at<double>(pl.dpat);
  q.qpat = db.at<double>(pl.qpat);
  q.qsh_o = db.at<double>(pl.qsh_o);
  q.qat_o = db.at<double>(pl.qat_o);
  q.dpat_o = db.at<double>(pl.dpat_o);
  q.qpat_o = db.at<double>(pl.qpat_o);
  q.vsh = db.at<double>(pl.vsh);
  q.vat = db.at<double>(pl.vat);
  q.vdp = db.at<double>(pl.vdp);
  q.vqp = db.at<double>(pl.vqp);
  q.vao = db.at<double>(pl.vao);
  q.mull = db.at<double>(pl.mull);
  q.eband = db.at<double>(pl.eband);
  q.eelec = db.at<double>(pl.eelec);
  q.erep = db.at<double>(pl.erep);
  q.vec_out = db.at<double>(pl.vec_out);
  q.scal = db.at<double>(pl.scal);
  q.icount = db.at<int>(pl.icount);
  q.bq = db.at<double>(pl.bq);
  q.bqlast = db.at<double>(pl.bqlast);
  q.bdq = db.at<double>(pl.bdq);
  q.bdqlast = db.at<double>(pl.bdqlast);
  q.bdf = db.at<double>(pl.bdf);
  q.bu = db.at<double>(pl.bu);
  q.ba = db.at<double>(pl.ba);
  q.bomega = db.at<double>(pl.bomega);
  q.bwork = db.at<double>(pl.bwork);
  q.bstatus = db.at<int>(pl.bstatus);
  q.grad = db.at<double>(pl.grad);
  q.sigma = db.at<double>(pl.sigma);
  q.sig_at = db.at<double>(pl.sig_at);
  q.dEdcn = db.at<double>(pl.dEdcn);
  q.X = db.at<double>(pl.X);
  q.A = db.at<double>(pl.A);
  q.T1 = db.at<double>(pl.T1);
  q.Y = db.at<double>(pl.Y);
  q.lu = db.at<double>(pl.lu);
  q.ed = db.at<double>(pl.ed);
  q.ee = db.at<double>(pl.ee);
  q.etau = db.at<double>(pl.etau);
  q.ew = nullptr;  // the batched eigenvalues go straight to emo
  q.epv = db.at<double>(pl.epv);
  q.escal = db.at<double>(pl.escal);
  q.estatus = db.at<int>(pl.estatus);
  q.conv = db.at<double>(pl.conv);
  q.param_grad = pl.param_grad ? 1 : 0;
  q.pgrad = pl.param_grad ? db.at<double>(pl.pgrad) : nullptr;
  q.zgrad = pl.param_grad ? db.at<double>(pl.zgrad) : nullptr;
  q.wbo_ch = pl.wbo_ch;
  q.wbo = pl.wbo_ch > 0 ? db.at<double>(pl.wbo) : nullptr;
  q.img = pl.sp2 ? db.at<uint16_t>(pl.img) : nullptr;
  q.iexp = pl.sp2 ? db.at<int>(pl.iexp) : nullptr;
  q.img2 = pl.sp2 ? db.at<uint16_t>(pl.img2) : nullptr;
  q.iexp2 = pl.sp2 ? db.at<int>(pl.iexp2) : nullptr;
  q.sp2s = pl.sp2 ? db.at<double>(pl.sp2s) : nullptr;
  q.sp2i = pl.sp2 ? db.at<int>(pl.sp2i) : nullptr;
  q.sp2p = pl.sp2 ? db.at<unsigned long long>(pl.sp2p) : nullptr;
  q.ximg[0] = pl.sp2 ? db.at<uint16_t>(pl.ximg0) : nullptr;
  q.ximg[1] = pl.sp2 ? db.at<uint16_t>(pl.ximg1) : nullptr;
  q.xexp[0] = pl.sp2 ? db.at<int>(pl.xexp0) : nullptr;
  q.xexp[1] = pl.sp2 ? db.at<int>(pl.xexp1) : nullptr;
  if (pl.sp2) q.nev = pl.nao;  // the projection needs no levels during the SCF; all after it
  return q;
}

// start charges (wavefunction/guess.f90:51-120): restart from a compatible result, else SAD
void start_charges(const Plan& pl, std::vector<double>& qsh, std::vector<double>& qat,
                   std::vector<double>& dp, std::vector<double>& qp) {
  const _tblite_calculator* c = pl.c;
  const _tblite_result* res = pl.res;
  const int nat = pl.nat, nsh = pl.nsh;
  if (res->has_wfn && res->nat == nat && res->nsh == nsh && res->nao == pl.nao) {
    qsh = res->qsh;
    qat = res->qat;
    dp = res->dpat;
    qp = res->qpat;
    return;
  }
  qsh.assign(nsh, 0.0);
  qat.assign(nat, pl.mol->charge / nat);
  dp.assign(3 * nat, 0.0);
  qp.assign(6 * nat, 0.0);
  std::vector<double> n0at(nat, 0.0);
  for (int i = 0; i < nsh; ++i) n0at[c->sh_atom[i]] += c->sh_refocc[i];
  for (int i = 0; i < nsh; ++i) qsh[i] = c->sh_refocc[i] / n0at[c->sh_atom[i]] * qat[c->sh_atom[i]];
}

// size buckets: consecutive molecules (sorted by orbital count, descending) while the count
// stays above 3/4 of the bucket's largest
std::vector<Bucket> make_buckets(const std::vector<Plan>& plans) {
  std::vector<Bucket> out;
  int i = 0;
  const int np = (int)plans.size();
  while (i < np) {
    Bucket b;
    b.first = i;
    b.sp2 = plans[i].sp2;
    const int top = plans[i].nao;
    int j = i;
    while (j < np && g_cut_den * plans[j].nao >= g_cut_num * top && j - i < 65535 &&
           plans[j].sp2 == b.sp2) {
      b.nat_max = std::max(b.nat_max, plans[j].nat);
      b.nsh_max = std::max(b.nsh_max, plans[j].nsh);
      b.nao_max = std::max(b.nao_max, plans[j].nao);
      b.nd_max = std::max(b.nd_max, plans[j].nd);
      ++j;
    }
    b.last = j;
    out.push_back(b);
    i = j;
  }
  return out;
}

struct Lists {
  std::vector<int> host;           // molecule indices, grouped by bucket
  std::vector<int> begin, count;   // per bucket
};

// one chunk of molecules through setup, SCF and gradient; fills results of the converged
// ones, returns the plan indices that must take the one-molecule path
std::vector<int> run_chunk(std::vector<Plan>& plans, Arena& ar, _tblite_context* ctx) {
  const auto t_stage = host_clock::now();
  const int np = (int)plans.size();
  Region R[NREG];
  for (auto& pl : plans) layout(pl, R);
  // molecule tables and launch lists live after the three regions
  Region tail;
  const size_t off_ptrs = tail.take(sizeof(MolPtrs) * np);
  const size_t off_list = tail.take(sizeof(int) * np);
  const size_t off_flag = tail.take(sizeof(int) * np);
  const size_t off_steps = tail.take(sizeof(int) * np);
  const size_t dbytes = R[RZ].size + R[RR].size + R[RS].size + R[RU].size + tail.size;
  const size_t hbytes = std::max(R[RU].size, R[RR].size) + tail.size;
  ar.reserve(dbytes, hbytes);
  cudaStream_t s = ar.stream;
  Bases db;
  db.base[RZ] = ar.dev;
  db.base[RR] = db.base[RZ] + R[RZ].size;
  db.base[RS] = db.base[RR] + R[RR].size;
  db.base[RU] = db.base[RS] + R[RS].size;
  char* dtail = db.base[RU] + R[RU].size;
  MolPtrs* d_ptrs = reinterpret_cast<MolPtrs*>(dtail + off_ptrs);
  int* d_list = reinterpret_cast<int*>(dtail + off_list);
  int* d_flag = reinterpret_cast<int*>(dtail + off_flag);
  int* d_steps = reinterpret_cast<int*>(dtail + off_steps);
  // host stage: uploaded region first, then the tables
  Bases hb{{nullptr, nullptr, nullptr, ar.host}};
  host_parallel(np, [&](int i) {
    const Plan& pl = plans[i];
    std::vector<double> qsh, qat, dp, qp;
    const _tblite_calculator* c = pl.c;
    stage(hb, pl.xyz, pl.mol->xyz);
    stage(hb, pl.at_z, c->at_z);
    stage(hb, pl.at_sh, c->at_sh);
    stage(hb, pl.sh_atom, c->sh_atom);
    stage(hb, pl.sh_l, c->sh_l);
    stage(hb, pl.sh_nprim, c->sh_nprim);
    stage(hb, pl.sh_alpha, c->sh_alpha);
    stage(hb, pl.sh_coeff, c->sh_coeff);
    stage(hb, pl.sh_ao, c->sh_ao);
    stage(hb, pl.ao_sh, c->ao_sh);
    stage(hb, pl.ao_at, c->ao_at);
    stage(hb, pl.sh_se0, c->sh_se0);
    stage(hb, pl.sh_kcn, c->sh_kcn);
    stage(hb, pl.sh_shpoly, c->sh_shpoly);
    stage(hb, pl.sh_zeta, c->sh_zeta);
    stage(hb, pl.sh_hub, c->sh_hub);
    stage(hb, pl.sh_gam3, c->sh_gam3);
    stage(hb, pl.sh_refocc, c->sh_refocc);
    stage(hb, pl.at_en, c->at_en);
    stage(hb, pl.at_rad, c->at_rad);
    stage(hb, pl.at_rcov, c->at_rcov);
    stage(hb, pl.at_mprad, c->at_mprad);
    stage(hb, pl.at_vcn, c->at_vcn);
    stage(hb, pl.at_dkern, c->at_dkern);
    stage(hb, pl.at_qkern, c->at_qkern);
    stage(hb, pl.at_repa, c->at_repa);
    stage(hb, pl.at_repz, c->at_repz);
    stage(hb, pl.sh_valence, c->sh_valence);
    stage(hb, pl.at_gam3, c->at_gam3);
    if (pl.has_d3) {
      stage(hb, pl.d3_nref, c->d3_nref);
      stage(hb, pl.d3_refcn, c->d3_refcn);
      stage(hb, pl.d3_sp, c->d3_sp);
      stage(hb, pl.d3_c6ref, c->d3_c6ref);
      stage(hb, pl.d3_r4r2, c->d3_r4r2);
      stage(hb, pl.d3_rcov, c->d3_rcov);
    }
    if (pl.has_d4) {
      stage(hb, pl.d4_sp, c->d4_sp);
      stage(hb, pl.d4_nref, c->d4_nref);
      stage(hb, pl.d4_ngw, c->d4_ngw);
      stage(hb, pl.d4_refcn, c->d4_refcn);
      stage(hb, pl.d4_refq, c->d4_refq);
      stage(hb, pl.d4_zeff, c->d4_zeff);
      stage(hb, pl.d4_gam, c->d4_gam);
      stage(hb, pl.d4_r4r2, c->d4_r4r2);
      stage(hb, pl.d4_rcov, c->d4_rcov);
      stage(hb, pl.d4_en, c->d4_en);
      stage(hb, pl.d4_c6ref, c->d4_c6ref);
    }
    start_charges(pl, qsh, qat, dp, qp);
    stage(hb, pl.qsh, qsh);
    stage(hb, pl.qat, qat);
    stage(hb, pl.dpat, dp);
    stage(hb, pl.qpat, qp);
  });
  cuda_check(cudaMemcpyAsync(db.base[RU], ar.host, R[RU].size, cudaMemcpyHostToDevice, s),
             "batch upload");
  cuda_check(cudaMemsetAsync(db.base[RZ], 0, R[RZ].size + R[RR].size, s), "batch zero");
  // molecule table (after the upload completes the stage can be reused)
  stream_wait(s);
  MolPtrs* h_ptrs = reinterpret_cast<MolPtrs*>(ar.host);
  for (int i = 0; i < np; ++i) {
    h_ptrs[i] = make_ptrs(plans[i], db);
    h_ptrs[i].flag = d_flag + i;
    h_ptrs[i].sp2steps = d_steps + i;
  }
  cuda_check(cudaMemcpyAsync(d_ptrs, h_ptrs, sizeof(MolPtrs) * np, cudaMemcpyHostToDevice, s),
             "batch table");
  cuda_check(cudaMemsetAsync(d_flag, 0, sizeof(int) * np, s), "flags");
  stream_wait(s);

  std::vector<Bucket> buckets = make_buckets(plans);
  const int nb = (int)buckets.size();
  std::vector<char> active(np, 1);
  std::vector<int> h_flag(np, 0);
  int* h_list = reinterpret_cast<int*>(ar.host);
  std::vector<BatchLaunch> launch(nb);
  auto upload_lists = [&](const std::vector<char>& sel) {
    int pos = 0;
    for (int bi = 0; bi < nb; ++bi) {
      const Bucket& b = buckets[bi];
      BatchLaunch& L = launch[bi];
      L.mp = d_ptrs;
      L.list = d_list + pos;
      L.nat_max = b.nat_max;
      L.nsh_max = b.nsh_max;
      L.nao_max = b.nao_max;
      L.nd_max = b.nd_max;
      L.sp2 = b.sp2 ? 1 : 0;
      L.sp2_steps = b.sp2_steps;
      L.s = s;
      int cnt = 0;
      for (int i = b.first; i < b.last; ++i)
        if (sel[i]) h_list[pos + cnt++] = i;
      L.count = cnt;
      pos += cnt;
    }
    if (pos)
      cuda_check(cudaMemcpyAsync(d_list, h_list, sizeof(int) * pos, cudaMemcpyHostToDevice, s),
                 "lists");
    stream_wait(s);  // the host list buffer is rewritten next time
    return pos;
  };
  // every bucket's steps on its own side stream (buckets touch disjoint molecules), ordered
  // after the work already on the main stream and joined back into it
  auto each = [&](auto&& fn) {
    cuda_check(cudaEventRecord(ar.fork, s), "fork");
    int k = 0;
    for (auto& L : launch) {
      if (!L.count) continue;
      const int slot = k++ % std::max(1, std::min(g_batch_streams, (int)Arena::NSIDE));
      L.s = ar.side[slot];
      cuda_check(cudaStreamWaitEvent(L.s, ar.fork, 0), "fork");
      fn(L);
      cuda_check(cudaEventRecord(ar.join[slot], L.s), "join");
      cuda_check(cudaStreamWaitEvent(s, ar.join[slot], 0), "join");
    }
  };
  const Gfn2Scalars p = gfn2_scalars(plans[0].c);  // h0_cutoff is taken per molecule
  bool any_sp2 = false;
  for (const Plan& pl : plans) any_sp2 = any_sp2 || pl.sp2;
  std::vector<int> h_steps(np, 0);
  bool any_param_grad = false;
  for (const Plan& pl : plans) any_param_grad = any_param_grad || pl.param_grad;

  // geometry setup
  upload_lists(active);
  cudaEvent_t ev0, ev1;
  cuda_check(cudaEventCreate(&ev0), "event");
  cuda_check(cudaEventCreate(&ev1), "event");
  cuda_check(cudaEventRecord(ev0, s), "event");
  g_last_host_ms[HP_STAGE] += ms_since(t_stage);
  each([&](BatchLaunch& L) {
    launch_cn_b(L, p);
    launch_setup_levels_b(L, p);
    launch_coulomb_table_b(L, p);  // needs the multipole radii of the levels kernel
    launch_build_h0_b(L, p);
    launch_repulsion_b(L, p);
    d4_setup_b(L);
    d3_setup_b(L);
    cholesky_inverse_b(L);
    if (L.sp2) pipe_x_images_b(L);  // X's slice images for the projection's products
  });
  cuda_check(cudaMemcpyAsync(h_flag.data(), d_flag, sizeof(int) * np, cudaMemcpyDeviceToHost, s),
             "flags");
  stream_wait(s);
  cuda_check(cudaGetLastError(), "batch setup");
  std::vector<int> leave;
  // why a molecule left the batch (recorded as a negative iteration count): -2 overlap not
  // positive definite, -1 singular Broyden system, -3 Fermi level above the computed levels,
  // -4 iteration limit or Broyden history
  auto record_leave = [&](int i, int code) {
    leave.push_back(i);
    if (plans[i].idx < (int)g_last_iters.size()) g_last_iters[plans[i].idx] = code;
  };
  for (int i = 0; i < np; ++i) {
    if (plans[i].c->fault == 1) h_flag[i] = -2;  // injected: overlap not positive definite
    if (h_flag[i] < 0) {
      active[i] = 0;
      record_leave(i, h_flag[i]);
    }
  }
  std::vector<char> done(np, 0);
  int max_iter = 0;
  for (auto& pl : plans) max_iter = std::max(max_iter, pl.max_iter);
  int iscf = 0;
  int nactive = upload_lists(active);
  auto t_iter = std::chrono::steady_clock::now();
  // every SCF iteration of the whole chunk (all buckets, all side streams) as one CUDA graph:
  // captured from the launch sequence, instantiated once and updated in place while the launch
  // structure stays the same (lists and step budgets change only as molecules converge), then
  // launched with one call; the per-kernel profiler's events are not captured, so a profiled
  // call launches the kernels directly
  const bool graphs = g_batch_graphs && !prof_enabled();
  cudaGraphExec_t gexec = nullptr;
  struct GraphGuard {
    cudaGraphExec_t* e;
    ~GraphGuard() {
      if (*e) cudaGraphExecDestroy(*e);
    }
  } gguard{&gexec};
  auto iteration = [&](auto&& body) {
    if (!graphs) {
      body();
      return;
    }
    cuda_check(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed), "capture");
    try {
      body();
    } catch (...) {
      cudaGraph_t dropped = nullptr;
      cudaStreamEndCapture(s, &dropped);
      if (dropped) cudaGraphDestroy(dropped);
      throw;
    }
    cudaGraph_t graph = nullptr;
    cuda_check(cudaStreamEndCapture(s, &graph), "capture");
    cudaGraphExecUpdateResultInfo info;
    if (!gexec || cudaGraphExecUpdate(gexec, graph, &info) != cudaSuccess) {
      cudaGetLastError();  // an update that does not fit is not an error: instantiate anew
      if (gexec) cudaGraphExecDestroy(gexec);
      gexec = nullptr;
      cuda_check(cudaGraphInstantiate(&gexec, graph, 0), "graph instantiate");
      ++g_last_graph_builds;
    }
    cudaGraphDestroy(graph);
    cuda_check(cudaGraphLaunch(gexec, s), "graph launch");
    ++g_last_graph_launches;
  };
  while (nactive > 0 && iscf < max_iter) {
    iteration([&]() {
    if (iscf > 0) {
      each([&](BatchLaunch& L) {
        launch_broyden_b(L, iscf);
        launch_unpack_b(L);
      });
    }
    each([&](BatchLaunch& L) {
      launch_coulomb_potential_b(L, p);
      d4_potential_b(L);
      launch_vao_b(L);
      launch_fock_b(L);
      launch_pack_b(L, false);
      if (L.sp2) {
        sp2_density_b(L, L.sp2_steps);
      } else {
        eigen_values_b(L);
        launch_fermi_b(L);
        eigen_vectors_b(L);
        density_b(L, false);
      }
      launch_mulliken_b(L);
      launch_pack_b(L, true);
      launch_diff_b(L);
      launch_eelec_init_b(L);
      launch_coulomb_energy_b(L, p);
      d4_energy_b(L);
      launch_converge_b(L);
    });
    });
    ++iscf;
    cuda_check(cudaMemcpyAsync(h_flag.data(), d_flag, sizeof(int) * np, cudaMemcpyDeviceToHost, s),
               "flags");
    if (any_sp2)
      cuda_check(cudaMemcpyAsync(h_steps.data(), d_steps, sizeof(int) * np, cudaMemcpyDeviceToHost,
                                 s),
                 "projection steps");
    stream_wait(s);
    cuda_check(cudaGetLastError(), "batch scf");
    // step budget of each projection bucket, set once after the first iteration: the most
    // steps its molecules took there plus a margin (the first, from the SAD guess, takes the
    // most); a fixed budget keeps the launch structure of the iteration graphs unchanged
    if (iscf == 1)
      for (Bucket& b : buckets) {
        if (!b.sp2) continue;
        int most = 0;
        for (int i = b.first; i < b.last; ++i)
          if (active[i]) most = std::max(most, h_steps[i]);
        b.sp2_steps = std::min(SP2_MAX_STEPS, most + 10);
      }
    for (int i = 0; i < np; ++i) {
      if (!active[i]) continue;
      const Plan& pl = plans[i];
      if (h_flag[i] == 1) {
        active[i] = 0;
        done[i] = 1;
        if (pl.idx < (int)g_last_iters.size()) g_last_iters[pl.idx] = iscf;
      } else if (h_flag[i] < 0 || iscf >= pl.max_iter ||
                 (iscf > HCAP && pl.memory > HCAP)) {
        active[i] = 0;
        record_leave(i, h_flag[i] < 0 ? h_flag[i] : -4);
      }
    }
    const int nbefore = nactive;
    nactive = upload_lists(active);
    if (ctx->verbosity > 1) {
      const auto now = std::chrono::steady_clock::now();
      char buf[160];
      snprintf(buf, sizeof(buf), "batch iteration %3d: %6d molecules, %6d still running, %9.3f ms",
               iscf, nbefore, nactive,
               std::chrono::duration<double, std::milli>(now - t_iter).count());
      ctx->message(buf);
      t_iter = now;
    }
  }
  for (int i = 0; i < np; ++i)
    if (active[i]) record_leave(i, -4);
  float scf_ms = 0.f;

  // projection buckets: every eigenvalue of the last Fock matrix (for the results) and the gap
  // check that makes their 0/2 occupations exact; a molecule below 80 kT leaves the batch
  if (any_sp2) {
    std::vector<char> sel(np, 0);
    for (int i = 0; i < np; ++i) sel[i] = done[i] && plans[i].sp2;
    if (upload_lists(sel) > 0) {
      each([&](BatchLaunch& L) {
        if (!L.sp2) return;
        eigen_values_b(L);
        launch_fermi_b(L);
        sp2_gap_b(L);
      });
      cuda_check(
          cudaMemcpyAsync(h_flag.data(), d_flag, sizeof(int) * np, cudaMemcpyDeviceToHost, s),
          "flags");
      stream_wait(s);
      cuda_check(cudaGetLastError(), "batch projection gap");
      for (int i = 0; i < np; ++i)
        if (sel[i] && h_flag[i] < 0) {
          done[i] = 0;
          record_leave(i, h_flag[i]);
        }
    }
  }

  // gradient of the converged molecules: Coulomb and D4 at the output moments, W into F,
  // H0 gradient with the last potential, CN chain rule
  if (upload_lists(done) > 0) {
    each([&](BatchLaunch& L) {
      if (!L.sp2) eigen_values_rest_b(L);  // the levels above the SCF's range, for the results
      launch_coulomb_gradient_b(L, p);
      d4_gradient_b(L);
      if (L.sp2) {
        sp2_weighted_b(L);  // W = P F P / 2
      } else {
        launch_fe_b(L);
        density_b(L, true);
      }
      launch_h0_gradient_b(L, p);
      launch_cn_grad_b(L, p);
      if (any_param_grad) {  // dE/d(shell parameters), Slater exponents (GFN2)
        launch_param_grad_b(L);
        launch_zeta_grad_b(L, p);
      }
    });
    // bond orders (post_processing/wbo.f90:60-115): closed shells from the total density,
    // restricted open shells per spin channel with the factor 2
    for (int ch = 0; ch < 2; ++ch) {
      std::vector<char> sel(np, 0);
      for (int i = 0; i < np; ++i) sel[i] = done[i] && plans[i].wbo_ch > ch;
      if (upload_lists(sel) > 0) each([&](BatchLaunch& L) { wbo_b(L, ch); });
    }
    if (any_sp2) {  // a pipelined product of the gradient phase whose wait ran out
      std::vector<char> sel(np, 0);
      for (int i = 0; i < np; ++i) sel[i] = done[i] && plans[i].sp2;
      if (upload_lists(sel) > 0) each([&](BatchLaunch& L) { sp2_pipe_check_b(L); });
    }
    cuda_check(cudaEventRecord(ev1, s), "event");
    cuda_check(cudaMemcpyAsync(ar.host, db.base[RR], R[RR].size, cudaMemcpyDeviceToHost, s),
               "batch results");
    cuda_check(cudaMemcpyAsync(h_flag.data(), d_flag, sizeof(int) * np, cudaMemcpyDeviceToHost, s),
               "flags");
    stream_wait(s);
    cuda_check(cudaGetLastError(), "batch gradient");
    // a split GEMM of the gradient phase that did not answer: the molecule is re-run by the
    // one-molecule path instead of reporting these results
    for (int i = 0; i < np; ++i)
      if (done[i] && h_flag[i] < 0) {
        done[i] = 0;
        record_leave(i, h_flag[i]);
      }
    cuda_check(cudaEventElapsedTime(&scf_ms, ev0, ev1), "event");
    const auto t_unpack = host_clock::now();
    const Bases hz{{nullptr, ar.host, nullptr, nullptr}};
    host_parallel(np, [&](int i) {
      if (!done[i]) return;
      const Plan& pl = plans[i];
      _tblite_result* res = pl.res;
      const int nat = pl.nat, n = pl.nao;
      auto get = [&](const Piece& pc, size_t count, std::vector<double>& out) {
        const double* src = hz.at<double>(pc);
        out.assign(src, src + count);
      };
      std::vector<double> eelec, erep, e3, sig_at, sigma;
      get(pl.eelec, nat, eelec);
      get(pl.erep, nat, erep);
      if (pl.has_d4) get(pl.d4_e3, nat, e3);
      res->nat = nat;
      res->nsh = pl.nsh;
      res->nao = n;
      res->energies.assign(nat, 0.0);
      res->energy = 0.0;
      for (int a = 0; a < nat; ++a) {
        double e = erep[a] + (pl.has_d4 ? e3[a] : 0.0);  // repulsion + three-body dispersion
        e += eelec[a];
        res->energies[a] = e;
        res->energy += e;
      }
      res->has_energy = true;
      get(pl.grad, 3 * nat, res->gradient);
      get(pl.sig_at, 9 * nat, sig_at);
      get(pl.sigma, 9, sigma);
      res->sigma.assign(9, 0.0);
      for (int k = 0; k < 9; ++k) {
        double acc = sigma[k];
        for (int a = 0; a < nat; ++a) acc += sig_at[9 * a + k];
        res->sigma[k] = acc;
      }
      get(pl.qsh_o, pl.nsh, res->qsh);
      get(pl.qat_o, nat, res->qat);
      get(pl.dpat_o, 3 * nat, res->dpat);
      get(pl.qpat_o, 6 * nat, res->qpat);
      get(pl.emo, n, res->emo);
      get(pl.focc, n, res->focc);
      res->P.clear();
      res->C.clear();
      res->S.clear();
      res->H.clear();
      res->wbo.clear();
      res->wbo_channels = pl.wbo_ch;
      if (pl.wbo_ch > 0) {
        get(pl.wbo, (size_t)pl.wbo_ch * nat * nat, res->wbo);
        if (pl.wbo_ch == 2) {  // (up, down) -> (total, magnetisation), wavefunction/spin.f90
          const size_t na2 = (size_t)nat * nat;
          for (size_t t = 0; t < na2; ++t) {
            const double up = res->wbo[t], dn = res->wbo[na2 + t];
            res->wbo[t] = up + dn;
            res->wbo[na2 + t] = up - dn;
          }
        }
      }
      res->has_wfn = true;
      molecular_moments(pl.mol, res);
      res->set_post_processing(pl.c->post_proc);
      if (pl.param_grad) {
        std::vector<double> pg;
        get(pl.pgrad, 4 * (size_t)pl.nsh, pg);
        const size_t ns = pl.nsh;
        res->dse.assign(pg.begin(), pg.begin() + ns);
        res->dhub.assign(pg.begin() + ns, pg.begin() + 2 * ns);
        res->dgam3.assign(pg.begin() + 2 * ns, pg.begin() + 3 * ns);
        res->dkcn.assign(pg.begin() + 3 * ns, pg.end());
        get(pl.zgrad, ns, res->dzeta);
      } else {
        res->dse.clear();
        res->dhub.clear();
        res->dgam3.clear();
        res->dkcn.clear();
        res->dzeta.clear();
      }
    });
    g_last_host_ms[HP_UNPACK] += ms_since(t_unpack);
  }
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  g_last_device_ms += scf_ms;
  return leave;
}

// device bytes one molecule needs in the batch (for chunking)
size_t molecule_bytes(const Plan& pl) {
  Plan tmp = pl;
  Region R[NREG];
  layout(tmp, R);
  return R[RZ].size + R[RR].size + R[RS].size + R[RU].size + sizeof(MolPtrs) + 64;
}

}  // namespace

extern "C" int tblite_gb300_batch_singlepoint(tblite_context ctx, int nmol,
                                              const tblite_structure* mols,
                                              const tblite_calculator* calcs,
                                              const tblite_result* results, int* status) {
  if (!ctx) return nmol;
  if (nmol <= 0) return 0;
  if (!mols || !calcs || !results) {
    ctx->push("Batch input arrays are missing");
    return nmol;
  }
  const auto t_call = host_clock::now();
  std::vector<int> st(nmol, 0);
  std::vector<Plan> plans;
  plans.reserve(nmol);
  std::vector<int> plain;  // molecules for the one-molecule path
  const int tri_max = batch_tridiag_max_n();
  for (int i = 0; i < nmol; ++i) {
    _tblite_calculator* c = calcs[i];
    const _tblite_structure* mol = mols[i];
    _tblite_result* res = results[i];
    if (!c || !mol || !res) {
      ctx->push("Batch entry " + std::to_string(i) + ": structure, calculator or result missing");
      st[i] = 1;
      continue;
    }
    if (mol->nat != c->nat) {
      ctx->push("Batch entry " + std::to_string(i) + ": structure does not match calculator");
      st[i] = 1;
      continue;
    }
    Plan pl{};
    pl.idx = i;
    pl.c = c;
    pl.mol = mol;
    pl.res = res;
    pl.nat = c->nat;
    pl.nsh = c->nsh;
    pl.nao = c->nao;
    pl.method = c->method;
    pl.nd = c->nsh + (c->method == 2 ? 9 * c->nat : 0);
    pl.max_iter = c->max_iter;
    pl.memory = c->memory > 0 ? std::min(c->memory, c->max_iter) : c->max_iter;
    pl.has_d4 = c->has_d4;
    pl.has_d3 = c->has_d3;
    try {
      electron_counts(c, mol, &pl.nalp, &pl.nbet);
    } catch (const std::exception& e) {
      ctx->push("Batch entry " + std::to_string(i) + ": " + e.what());
      st[i] = 1;
      continue;
    }
    const bool anneal = c->anneal && c->anneal_kt > c->etemp;
    // implicit solvation and an electric field run on the one-molecule path
    pl.param_grad = c->param_grad != 0;
    c->default_post_processing();  // as a plain single point does
    pl.wbo_ch = c->wants("bond-orders") ? (pl.nalp != pl.nbet ? 2 : 1) : 0;
    pl.molmom = c->wants("molmom");
    // the projection needs a closed shell with a whole number of electron pairs
    pl.sp2 = g_batch_sp2 && pl.nao >= g_sp2_min_nao && pl.nalp == pl.nbet &&
             pl.nalp == std::floor(pl.nalp) && pl.nalp >= 1.0;
    if (pl.nao > tri_max || anneal || pl.max_iter < 1 || c->solv || c->has_field) {
      plain.push_back(i);
      continue;
    }
    plans.push_back(pl);
  }
  // one chunk runs one Hamiltonian: the plans are grouped by their global model constants
  // (GFN2-xTB, GFN1-xTB, IPEA1-xTB or a custom record of either form), then largest first;
  // the size buckets follow the sorted order
  {
    std::vector<std::pair<int, const ModelConstants*>> models;  // (method, constants)
    for (Plan& pl : plans) {
      const ModelConstants& m = pl.c->model;
      int id = -1;
      for (size_t k = 0; k < models.size() && id < 0; ++k)
        if (models[k].first == pl.method && same_model(*models[k].second, m)) id = (int)k;
      if (id < 0) {
        id = (int)models.size();
        models.push_back({pl.method, &m});
      }
      pl.model = id;
    }
  }
  {  // sorted through an index permutation: a plan holds ~140 array offsets
    std::vector<int> order(plans.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int i, int j) {
      const Plan& a = plans[i];
      const Plan& b = plans[j];
      if (a.model != b.model) return a.model < b.model;
      if (a.sp2 != b.sp2) return a.sp2;
      return a.nao > b.nao;
    });
    std::vector<Plan> sorted;
    sorted.reserve(plans.size());
    for (int k : order) sorted.push_back(plans[k]);
    plans.swap(sorted);
  }
  try {
    std::lock_guard<std::mutex> lock(g_batch_mutex);
    for (double& t : g_last_host_ms) t = 0.0;
    g_last_host_ms[HP_PLAN] = ms_since(t_call);
    g_last_device_ms = 0.0;
    g_last_projected = 0;
    g_last_graph_builds = g_last_graph_launches = 0;
    g_last_iters.assign(nmol, 0);
    g_last_modes.assign(nmol, -1);
    prof_reset();
    // chunks of at most ~24 GB of device memory
    const size_t budget = (size_t)24 << 30;
    size_t i0 = 0;
    std::vector<size_t> mbytes(plans.size());
    {
      const auto t_chunk = host_clock::now();
      for (size_t k = 0; k < plans.size(); ++k) mbytes[k] = molecule_bytes(plans[k]);
      g_last_host_ms[HP_CHUNK] = ms_since(t_chunk);
    }
    while (i0 < plans.size()) {
      size_t i1 = i0, bytes = 0;
      while (i1 < plans.size() && plans[i1].model == plans[i0].model &&
             (i1 == i0 || bytes + mbytes[i1] <= budget)) {
        bytes += mbytes[i1];
        ++i1;
      }
      std::vector<Plan> chunk(plans.begin() + i0, plans.begin() + i1);
      const std::vector<int> leave = run_chunk(chunk, g_arena, ctx);
      for (int k : leave) plain.push_back(chunk[k].idx);
      std::vector<char> left(chunk.size(), 0);
      for (int k : leave) left[k] = 1;
      for (size_t k = 0; k < chunk.size(); ++k) {
        g_last_projected += chunk[k].sp2 && !left[k];
        if (!left[k]) g_last_modes[chunk[k].idx] = chunk[k].sp2 ? 1 : 0;
      }
      i0 = i1;
    }
    prof_collect();
  } catch (const std::exception& e) {
    ctx->push(std::string("batched single points failed: ") + e.what());
    for (int i = 0; i < nmol; ++i) st[i] = 1;
    if (status)
      for (int i = 0; i < nmol; ++i) status[i] = st[i];
    return nmol;
  }
  // the one-molecule path for the rest (reproduces a plain call, errors included)
  std::sort(plain.begin(), plain.end());
  g_last_fallbacks = (int)plain.size();
  const auto t_plain = host_clock::now();
  for (int i : plain) {
    try {
      run_singlepoint(ctx, mols[i], calcs[i], results[i]);
    } catch (const std::exception& e) {
      ctx->push("Batch entry " + std::to_string(i) + ": " + e.what());
      st[i] = 1;
    }
  }
  g_last_host_ms[HP_PLAIN] = ms_since(t_plain);
  g_last_host_ms[HP_TOTAL] = ms_since(t_call);
  int failed = 0;
  for (int i = 0; i < nmol; ++i) failed += st[i];
  if (status)
    for (int i = 0; i < nmol; ++i) status[i] = st[i];
  return failed;
}

extern "C" int tblite_gb300_batch_last_fallbacks(void) { return g_last_fallbacks; }
extern "C" void tblite_gb300_set_split_gemm(int enable) { tb::g_split_gemm = enable != 0; }
namespace tb {
void set_tridiag_ctas_per_sm(int k);
void set_tridiag_small(int k);
}
extern "C" void tblite_gb300_set_small_tridiag(int full_storage) {
  tb::set_tridiag_small(full_storage);
}
extern "C" void tblite_gb300_set_tridiag_ctas_per_sm(int count) {
  tb::set_tridiag_ctas_per_sm(count);
}
extern "C" void tblite_gb300_set_batch_density_solver(int mode) { g_batch_sp2 = mode != 0; }
extern "C" int tblite_gb300_batch_last_projected(void) { return g_last_projected; }
extern "C" int tblite_gb300_batch_last_modes(int* modes, int nmol) {
  const int m = std::min(nmol, (int)g_last_modes.size());
  for (int i = 0; i < m && modes; ++i) modes[i] = g_last_modes[i];
  return (int)g_last_modes.size();
}
extern "C" void tblite_gb300_set_batch_graphs(int enable) { g_batch_graphs = enable != 0; }
extern "C" int tblite_gb300_batch_last_graphs(int* builds, int* launches) {
  if (builds) *builds = g_last_graph_builds;
  if (launches) *launches = g_last_graph_launches;
  return g_batch_graphs ? 1 : 0;
}
extern "C" void tblite_gb300_set_batch_streams(int count) {
  g_batch_streams = count < 1 ? 1 : (count > Arena::NSIDE ? Arena::NSIDE : count);
}
extern "C" int tblite_gb300_set_projection_threshold(int nao) {
  const int old = g_sp2_min_nao;
  if (nao > 0) g_sp2_min_nao = nao;
  return old;
}
extern "C" double tblite_gb300_batch_last_device_ms(void) { return g_last_device_ms; }
extern "C" int tblite_gb300_batch_last_host_ms(double* ms, int n) {
  const int m = std::min(n, (int)HP_N);
  for (int k = 0; k < m && ms; ++k) ms[k] = g_last_host_ms[k];
  return HP_N;
}
extern "C" int tblite_gb300_batch_last_iterations(int* iterations, int nmol) {
  const int m = std::min(nmol, (int)g_last_iters.size());
  for (int i = 0; i < m && iterations; ++i) iterations[i] = g_last_iters[i];
  return (int)g_last_iters.size();
}

namespace tb {
int get_tridiag_ctas_per_sm();
int get_tridiag_small();
}

// back to the default schedule (CUDA graphs, projection from 96 orbitals, bucket cut 3/4, two
// CTAs per SM, full-storage small tridiagonalisation, 8 streams)
extern "C" void tblite_gb300_batch_reset_schedule(void) {
  g_batch_graphs = true;
  g_sp2_min_nao = SP2_MIN_NAO;
  g_cut_num = 3;
  g_cut_den = 4;
  tb::set_tridiag_ctas_per_sm(2);
  tb::set_tridiag_small(1);
  g_batch_streams = 8;
  g_schedule_note = "defaults";
}

// The batch schedule: projection threshold, bucket cut, CTAs per SM of the cluster
// tridiagonalisation and side streams, as a short text for logs and benchmark records.
extern "C" int tblite_gb300_batch_schedule(char* buf, int n) {
  char tmp[384];
  const int len = std::snprintf(
      tmp, sizeof(tmp),
      "projection from %d orbitals%s; bucket cut %d/%d; tridiagonalisation %d CTA(s) per SM, "
      "%s below 157 orbitals; %d streams; %s",
      g_sp2_min_nao, g_batch_sp2 ? "" : " (off)", g_cut_num, g_cut_den,
      tb::get_tridiag_ctas_per_sm(), tb::get_tridiag_small() ? "full storage" : "packed",
      g_batch_streams, g_schedule_note.c_str());
  if (buf && n > 0) {
    std::strncpy(buf, tmp, (size_t)n - 1);
    buf[n - 1] = '\0';
  }
  return len;
}

// Autotuner of the batch schedule (no counterpart in the reference): coordinate descent over
// CUDA graphs on/off, the projection threshold, the bucket cut, the CTAs per SM of the tridiagonalisation and the side
// streams, each candidate timed (wall time of the call, best of three) on a seeded sample of the given
// molecules; the fastest schedule stays set.  Returns the number of timed calls, or -1 if the
// sample could not be evaluated (the schedule is then left as it was).
extern "C" int tblite_gb300_batch_autotune(tblite_context ctx, int nmol,
                                           const tblite_structure* mols,
                                           const tblite_calculator* calcs, int sample) {
  if (!ctx || nmol <= 0 || !mols || !calcs) return -1;
  std::vector<int> idx(nmol);
  std::iota(idx.begin(), idx.end(), 0);
  unsigned long long state = 0x9E3779B97F4A7C15ull;  // fixed seed: the same sample every time
  for (int i = nmol - 1; i > 0; --i) {             // Fisher-Yates with a 64-bit LCG
    state = state * 6364136223846793005ull + 1442695040888963407ull;
    std::swap(idx[i], idx[(int)((state >> 33) % (unsigned long long)(i + 1))]);
  }
  const int k = std::max(1, std::min(nmol, sample > 0 ? sample : 256));
  std::vector<tblite_structure> sm(k);
  std::vector<tblite_calculator> sc(k);
  std::vector<_tblite_result> rs(k);
  std::vector<tblite_result> sr(k);
  for (int i = 0; i < k; ++i) {
    sm[i] = mols[idx[i]];
    sc[i] = calcs[idx[i]];
    sr[i] = &rs[i];
  }
  _tblite_context quiet;
  quiet.verbosity = 0;
  int calls = 0;
  auto time_it = [&]() {
    double best = 1e300;
    for (int r = 0; r < 3; ++r) {
      quiet.errors.clear();
      // wall time of the whole call: molecules handed to the one-molecule path count too
      const auto t0 = std::chrono::steady_clock::now();
      if (tblite_gb300_batch_singlepoint(&quiet, k, sm.data(), sc.data(), sr.data(), nullptr) != 0)
        return -1.0;
      const auto t1 = std::chrono::steady_clock::now();
      ++calls;
      best = std::min(best, std::chrono::duration<double, std::milli>(t1 - t0).count());
    }
    return best;
  };
  const int sp2_keep = g_sp2_min_nao, num_keep = g_cut_num, den_keep = g_cut_den,
            ctas_keep = tb::get_tridiag_ctas_per_sm(), streams_keep = g_batch_streams;
  double best = time_it();
  if (best < 0) return -1;
  // a candidate replaces the current choice only when more than 1 % faster (the calls' timing
  // noise is of that order)
  auto try_values = [&](auto set, const std::vector<int>& values, int& keep) {
    for (int v : values) {
      if (v == keep) continue;
      set(v);
      const double t = time_it();
      if (t >= 0 && t < 0.99 * best) {
        best = t;
        keep = v;
      }
    }
    set(keep);
  };
  int sp2 = sp2_keep, cut = num_keep * 10 + den_keep, ctas = ctas_keep, streams = streams_keep;
  // CUDA graphs first (only switched off, never on against the caller's setting): a projection
  // iteration is a long launch sequence whose graph is instantiated again whenever its step
  // budget changes, which can cost more than the launches it saves
  int graphs = g_batch_graphs ? 1 : 0;
  if (graphs) try_values([](int v) { g_batch_graphs = v != 0; }, {0}, graphs);
  try_values([](int v) { g_sp2_min_nao = v; }, {64, 80, 96, 112, 128, 144, 176, 100000}, sp2);
  try_values([](int v) { g_cut_num = v / 10; g_cut_den = v % 10; }, {34, 23, 45}, cut);
  try_values([](int v) { tb::set_tridiag_ctas_per_sm(v); }, {1, 2}, ctas);
  int small = tb::get_tridiag_small();
  try_values([](int v) { tb::set_tridiag_small(v); }, {0, 1}, small);
  try_values([](int v) { g_batch_streams = v; }, {4, 8, 16}, streams);
  char note[160];
  std::snprintf(note, sizeof(note), "autotuned on %d molecules (%d calls, %.1f ms)%s", k, calls,
                best, g_batch_graphs ? "" : "; SCF iterations launched directly");
  g_schedule_note = note;
  return calls;
}
