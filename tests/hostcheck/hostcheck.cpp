// Host build of the kernels' arithmetic (field, curve, recovery, tables) for
// the CPU test tier: the carry flag is emulated (arith.cuh), everything else is
// the exact source the sm_103a kernels compile.  Test-only; never linked into
// the library.
#include <string.h>
#include "../../wgpu-sigops_gb300/csrc/tables.cuh"
#include "../../wgpu-sigops_gb300/csrc/serve_policy.h"

using namespace sg;

static const uint32_t *g_k1, *g_r1, *g_ed;

static void init() {
  const KernelTables& t = kernel_tables();
  g_k1 = t.tab[CURVE_SECP256K1].data();
  g_r1 = t.tab[CURVE_SECP256R1].data();
  g_ed = t.tab[CURVE_ED25519].data();
}

static u256 load_le(const uint8_t* b) { u256 r; memcpy(r.w, b, 32); return r; }
static void store_le(const u256& v, uint8_t* b) { memcpy(b, v.w, 32); }

extern "C" {

int hc_bases(int curve, uint32_t L, uint32_t* out) { return build_bases(curve, L, out); }

// entries of the generator tables: ECDSA (per half for secp256k1), ed25519
int hc_gtab_entries(int ed) { return ed ? ED_GTAB : ECDSA_GTAB; }

void hc_gtab(int curve, uint32_t* out) {
  init();
  if (curve == 0) memcpy(out, g_k1, 2 * ECDSA_GTAB * 16 * 4);
  else if (curve == 1) memcpy(out, g_r1, ECDSA_GTAB * 16 * 4);
  else memcpy(out, g_ed, ED_GTAB * 24 * 4);
}

// field op test: field 0 k1-p, 1 r1-p, 2 ed-p, 3 k1-n, 4 r1-n, 5 ed-l ; op 0 mul, 1 add, 2 sub, 3 inv, 4 sqrt_candidate/pow_p58
// integers little-endian; inputs < modulus
void hc_field(int field, int op, const uint8_t* a, const uint8_t* b, uint8_t* out) {
  u256 x = load_le(a), y = load_le(b), r = u256_zero();
#define OPS(F)                                                        \
  {                                                                   \
    u256 xa = F::from_int(x), ya = F::from_int(y), ra;                \
    if (op == 0) ra = F::mul(xa, ya);                                 \
    else if (op == 1) ra = F::add(xa, ya);                            \
    else if (op == 2) ra = F::sub(xa, ya);                            \
    else ra = F::inv(xa);                                             \
    r = F::to_int(ra);                                                \
  }
  switch (field) {
    case 0: if (op == 4) r = FpK1::to_int(FpK1::sqrt_candidate(FpK1::from_int(x))); else OPS(FpK1); break;
    case 1: if (op == 4) r = FpR1::to_int(FpR1::sqrt_candidate(FpR1::from_int(x))); else OPS(FpR1); break;
    case 2: if (op == 4) r = FpEd::canon(FpEd::pow_p58(FpEd::from_int(x))); else OPS(FpEd); break;
    case 3: if (op == 5) r = ScK1::inv_int(x); else OPS(ScK1); break;  // op 5: the kernels' r^-1 (divsteps, checked)
    case 4: if (op == 5) r = ScR1::inv_int(x); else OPS(ScR1); break;
    case 5: OPS(ScEd); break;
  }
#undef OPS
  store_le(r, out);
}

void hc_mul_wide(const uint8_t* a, const uint8_t* b, uint8_t* out64) {
  uint32_t t[16];
  mul_wide(t, load_le(a), load_le(b));
  memcpy(out64, t, 64);
}

// which = 0: schoolbook, 1: Karatsuba
void hc_mul_wide_form(int which, const uint8_t* a, const uint8_t* b, uint8_t* out64) {
  uint32_t t[16];
  if (which) mul_wide_kara(t, load_le(a), load_le(b));
  else mul_wide_school(t, load_le(a), load_le(b));
  memcpy(out64, t, 64);
}

int hc_k1_recover(const uint8_t* sig, const uint8_t* msg, uint8_t* out) {
  init();
  uint32_t s[16], m[8], o[16];
  memcpy(s, sig, 64); memcpy(m, msg, 32);
  int st = ecdsa_recover<K1Traits>(s, m, g_k1, o);
  memcpy(out, o, 64);
  return st;
}

int hc_r1_recover(const uint8_t* sig, const uint8_t* msg, uint8_t* out) {
  init();
  uint32_t s[16], m[8], o[16];
  memcpy(s, sig, 64); memcpy(m, msg, 32);
  int st = ecdsa_recover<R1Traits>(s, m, g_r1, o);
  memcpy(out, o, 64);
  return st;
}

int hc_ed_verify(const uint8_t* sig, const uint8_t* msg, const uint8_t* pk) {
  init();
  uint32_t s[16], m[8], p[8];
  memcpy(s, sig, 64); memcpy(m, msg, 32); memcpy(p, pk, 32);
  return ed25519_verify(s, m, p, g_ed);
}

int hc_ed_verify_raw(const uint8_t* sig, const uint8_t* msg, uint32_t len, const uint8_t* pk) {
  init();
  uint32_t s[16], p[8];
  memcpy(s, sig, 64); memcpy(p, pk, 32);
  return ed25519_verify_raw(s, msg, len, p, g_ed);
}

void hc_sha512_96(const uint8_t* in, uint8_t* out) {
  uint32_t m[24], h[16];
  memcpy(m, in, 96);
  sha512_96(m, h);
  memcpy(out, h, 64);
}

}  // extern "C"

#include "../../wgpu-sigops_gb300/csrc/sign.cuh"

extern "C" int hc_ecdsa_sign(int curve, const uint8_t* d, const uint8_t* k, const uint8_t* msg, uint8_t* sig, uint8_t* pub) {
  init();
  uint32_t dw[8], kw[8], m[8], s[16], p[16];
  memcpy(dw, d, 32); memcpy(kw, k, 32); memcpy(m, msg, 32);
  int st = curve == 0 ? ecdsa_sign<K1Traits>(dw, kw, m, g_k1, s, p) : ecdsa_sign<R1Traits>(dw, kw, m, g_r1, s, p);
  memcpy(sig, s, 64); memcpy(pub, p, 64);
  return st;
}

extern "C" void hc_ed_sign(const uint8_t* seed, const uint8_t* msg, uint8_t* sig, uint8_t* pk) {
  init();
  uint32_t sd[8], m[8], s[16], p[8];
  memcpy(sd, seed, 32); memcpy(m, msg, 32);
  ed25519_sign(sd, m, g_ed, s, p);
  memcpy(sig, s, 64); memcpy(pk, p, 32);
}

// weakly reduced field operations (field 0 secp256k1, 1 P-256, 2 ed25519)
// on raw inputs below 2^256, raw result: op 0 add, 1 sub, 2 mul, 3 sqr,
// 4 neg, 5 is_zero, 6 half (5 and 6: secp256k1, P-256)
template <class F>
static u256 weak_op(int op, const u256& x, const u256& y) {
  if (op == 0) return F::add(x, y);
  if (op == 1) return F::sub(x, y);
  if (op == 2) return F::mul(x, y);
  if (op == 3) return F::sqr(x);
  return F::neg(x);
}
extern "C" void hc_weak(int field, int op, const uint8_t* a, const uint8_t* b, uint8_t* out) {
  u256 x = load_le(a), y = load_le(b), r = u256_zero();
  if (op == 5) r.w[0] = field == 0 ? FpK1::is_zero(x) : FpR1::is_zero(x);
  else if (op == 6) r = field == 0 ? FpK1::half(x) : FpR1::half(x);
  else if (field == 0) r = weak_op<FpK1>(op, x, y);
  else if (field == 1) r = weak_op<FpR1>(op, x, y);
  else r = weak_op<FpEd>(op, x, y);
  store_le(r, out);
}

// x < 2^256 into the field's canonical range (from_int); field 0 k1, 1 r1, 2 ed
extern "C" void hc_canon(int field, const uint8_t* x, uint8_t* out) {
  u256 v = load_le(x), r;
  if (field == 0) r = FpK1::from_int(v);
  else if (field == 1) r = FpR1::to_int(FpR1::from_int(v));
  else r = FpEd::canon(v);
  store_le(r, out);
}

// Weierstrass point operations on Jacobian inputs built from affine points and
// chosen Z: P = (x z^2, y z^3, z) (z = 0: infinity).  op 0: add(P, Q),
// 1: madd(P, Q affine), 2: dbl(P).  out = affine x || y, returns 1 for the
// point at infinity.
template <class T>
static int weier_op(int op, const uint8_t* pa, const uint8_t* pz, const uint8_t* qa, const uint8_t* qz, uint8_t* out) {
  using F = typename T::F;
  using W = Weier<F, T::A_M3>;
  auto jac = [](const uint8_t* a, const uint8_t* zb) {
    JPoint r;
    const u256 z = F::from_int(load_le(zb));
    if (u256_is_zero(z)) return W::infinity();
    const u256 x = F::from_int(load_le(a)), y = F::from_int(load_le(a + 32)), z2 = F::sqr(z);
    r.X = F::mul(x, z2);
    r.Y = F::mul(y, F::mul(z2, z));
    r.Z = z;
    return r;
  };
  JPoint P = jac(pa, pz), R;
  if (op == 0) R = W::add(P, jac(qa, qz));
  else if (op == 1) {
    APoint q;
    q.x = F::from_int(load_le(qa));
    q.y = F::from_int(load_le(qa + 32));
    R = W::madd(P, q);
  } else R = W::dbl(P);
  if (W::is_inf(R)) return 1;
  APoint a = W::to_affine(R);
  store_le(F::to_int(a.x), out);
  store_le(F::to_int(a.y), out + 32);
  return 0;
}

extern "C" int hc_weier_op(int curve, int op, const uint8_t* pa, const uint8_t* pz, const uint8_t* qa, const uint8_t* qz, uint8_t* out) {
  return curve == 0 ? weier_op<K1Traits>(op, pa, pz, qa, qz, out) : weier_op<R1Traits>(op, pa, pz, qa, qz, out);
}

// P-256 reduction of a 512-bit value
extern "C" void hc_r1_reduce(const uint8_t* x64, uint8_t* out) {
  uint32_t t[16];
  memcpy(t, x64, 64);
  store_le(FpR1::reduce(t), out);
}

// reduction of a 512-bit value in field 0 (secp256k1), 1 (P-256), 2 (ed25519)
extern "C" void hc_reduce(int field, const uint8_t* x64, uint8_t* out) {
  uint32_t t[16];
  memcpy(t, x64, 64);
  store_le(field == 0 ? FpK1::reduce(t) : field == 1 ? FpR1::reduce(t) : FpEd::reduce(t), out);
}

// multiply instructions counted since the last reset (this thread)
extern "C" uint64_t hc_mulcount(int reset) {
  const uint64_t c = mulcount_();
  if (reset) mulcount_() = 0;
  return c;
}

extern "C" void hc_sqr_wide(const uint8_t* a, uint8_t* out64) {
  uint32_t t[16];
  u256 x;
  memcpy(x.w, a, 32);
  sqr_wide(t, x);
  memcpy(out64, t, 64);
}

extern "C" int hc_k1_recover_glv(const uint8_t* sig, const uint8_t* msg, uint8_t* out) {
  init();
  uint32_t s[16], m[8], o[16];
  memcpy(s, sig, 64); memcpy(m, msg, 32);
  int st = ecdsa_recover<K1Traits, true>(s, m, g_k1, o);
  memcpy(out, o, 64);
  return st;
}

#include "../../wgpu-sigops_gb300/csrc/inverse.cuh"

// x^-1 mod M by divsteps; *batches_used = first batch after which g == 0
extern "C" void hc_divstep_inv(const uint8_t* x, const uint8_t* m, uint32_t minv30, uint8_t* out, int* batches_used) {
  u256 xv = load_le(x), mv = load_le(m);
  store_le(divstep_inverse(xv, mv, minv30), out);
  // count batches until g == 0
  S30 M = s30_from_u256(mv), f = M, g = s30_from_u256(xv), d, e;
  for (int i = 0; i < 9; ++i) { d.v[i] = 0; e.v[i] = 0; }
  e.v[0] = 1;
  int32_t delta2 = 1;
  int used = -1;
  for (int it = 0; it < DIVSTEP_BATCHES; ++it) {
    int32_t t[4];
    delta2 = divsteps30(delta2, (uint32_t)f.v[0] | ((uint32_t)f.v[1] << 30), (uint32_t)g.v[0] | ((uint32_t)g.v[1] << 30), t);
    s30_update_de(d, e, t, M, minv30);
    s30_update_fg(f, g, t);
    bool zero = true;
    for (int k = 0; k < 9; ++k) zero &= g.v[k] == 0;
    if (zero && used < 0) used = it + 1;
  }
  *batches_used = used;
}

// The batched engine's single-curve path with its shared inversions, on the
// host: one curve's n items, thread t of T = ceil(n / batch) taking items
// t, t + T, ... as rinv_kernel / finish_kernel do; r^-1 by simultaneous
// inversion, the curve step to the projective result, then the simultaneous
// inversion of Z and the key bytes (ECDSA) or the R comparison (ed25519).
// out: n x 64 mixed records, status: n.
template <class T, bool GLV>
static void deferred_ecdsa(const uint8_t* sigs, const uint8_t* msgs, size_t n, int batch, const uint32_t* gtab, uint8_t* out,
                           uint8_t* status) {
  using S = typename T::S;
  using F = typename T::F;
  const size_t nt = (n + batch - 1) / batch;
  std::vector<u256> rinv(n), v(batch), pre(batch);
  std::vector<JPoint> q(n);
  for (size_t t = 0; t < nt; ++t) {
    int m = 0;
    for (; m < batch && t + m * nt < n; ++m) {
      uint32_t s[16];
      memcpy(s, sigs + 64 * (t + m * nt), 64);
      v[m] = ecdsa_r_factor<T>(s);
    }
    batch_invert<S>(v.data(), pre.data(), m, [](const u256& x) { return S::from_int(S::inv_int(S::to_int(x))); });
    for (int j = 0; j < m; ++j) rinv[t + j * nt] = v[j];
  }
  for (size_t i = 0; i < n; ++i) {
    uint32_t s[16], mw[8];
    memcpy(s, sigs + 64 * i, 64);
    memcpy(mw, msgs + 32 * i, 32);
    u256 r, sv, z;
    APoint R;
    uint8_t st = ecdsa_prepare<T>(s, mw, r, sv, z, R);
    if (st == ST_OK) st = ecdsa_key_jacobian<T, GLV>(sv, z, R, rinv[i], gtab, q[i]);
    status[i] = st;
    memset(out + 64 * i, 0, 64);
  }
  std::vector<size_t> item(batch);
  for (size_t t = 0; t < nt; ++t) {
    int m = 0;
    for (int j = 0; j < batch && t + j * nt < n; ++j) {
      const size_t i = t + j * nt;
      if (status[i] != ST_OK) continue;
      item[m] = i;
      v[m++] = q[i].Z;
    }
    if (!m) continue;
    batch_invert<F>(v.data(), pre.data(), m, [](const u256& x) { return F::inv(x); });
    for (int j = 0; j < m; ++j) {
      uint32_t o[16];
      ecdsa_encode_key<T>(q[item[j]], v[j], o);
      memcpy(out + 64 * item[j], o, 64);
    }
  }
}

static void deferred_ed(const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks, size_t n, int batch, uint8_t* out, uint8_t* status) {
  const size_t nt = (n + batch - 1) / batch;
  std::vector<EPoint> rp(n);
  std::vector<u256> v(batch), pre(batch);
  for (size_t i = 0; i < n; ++i) {
    uint32_t s[16], mw[8], p[8];
    memcpy(s, sigs + 64 * i, 64);
    memcpy(mw, msgs + 32 * i, 32);
    memcpy(p, pks + 32 * i, 32);
    status[i] = ed25519_point(s, mw, p, g_ed, rp[i]);
    memset(out + 64 * i, 0, 64);
  }
  std::vector<size_t> item(batch);
  for (size_t t = 0; t < nt; ++t) {
    int m = 0;
    for (int j = 0; j < batch && t + j * nt < n; ++j) {
      const size_t i = t + j * nt;
      if (status[i] != ST_OK) continue;
      item[m] = i;
      v[m++] = rp[i].Z;
    }
    if (!m) continue;
    batch_invert<FpEd>(v.data(), pre.data(), m, [](const u256& x) { return FpEd::inv(x); });
    for (int j = 0; j < m; ++j) {
      uint32_t s[16];
      memcpy(s, sigs + 64 * item[j], 64);
      status[item[j]] = ed25519_compare(rp[item[j]], v[j], s);
      out[64 * item[j]] = status[item[j]] == ST_OK;
    }
  }
}

extern "C" void hc_batched_deferred(int curve, const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks, size_t n, int batch,
                                    uint8_t* out, uint8_t* status) {
  init();
  if (curve == 0) deferred_ecdsa<K1Traits, true>(sigs, msgs, n, batch, g_k1, out, status);
  else if (curve == 1) deferred_ecdsa<R1Traits, false>(sigs, msgs, n, batch, g_r1, out, status);
  else deferred_ed(sigs, msgs, pks, n, batch, out, status);
}

// The serving loop's adaptive shape (serve_policy.h) over simulated arrivals:
// a dispatcher that looks every step_s seconds, items_cum[i] = items accepted
// by step i.  shapes[i] = the shape a launch at step i would take (a shape
// switch needs a relaunch; here every step counts as one), rates[i] = the
// estimate.  switch_rate 0 = the fixed shape.
extern "C" void hc_shape_policy_run(int low, int high, double switch_rate, int fixed, const uint64_t* items_cum, int steps, double step_s,
                                    int* shapes, double* rates) {
  sg::ShapePolicy p;
  p.low = low;
  p.high = high;
  p.switch_rate = switch_rate;
  int running = p.wanted(fixed, fixed);
  for (int i = 0; i < steps; ++i) {
    p.observe((i + 1) * step_s, items_cum[i]);
    running = p.wanted(fixed, running);
    shapes[i] = running;
    rates[i] = p.rate;
  }
}

// coz_table_iso against coz_table for the secp256k1 point R = (x, y) (32-byte
// little-endian integers): entry k of the first, at the common Z zc, must be
// the affine entry k of the second mapped by (x, y) -> (x zc^2, y zc^3).
// Returns the number of coordinates that differ (0..32).
extern "C" int hc_coz_iso_mismatches(const uint8_t* x_le, const uint8_t* y_le) {
  using F = FpK1;
  constexpr int NR = 16;
  APoint R;
  R.x = F::from_int(load_le(x_le));
  R.y = F::from_int(load_le(y_le));
  APoint aff[NR], iso[NR];
  u256 zc;
  coz_table<F, false, NR>(R, aff);
  coz_table_iso<F, NR>(R, iso, zc);
  const u256 z2 = F::sqr(zc), z3 = F::mul(z2, zc);
  int bad = 0;
  for (int k = 0; k < NR; ++k) {
    bad += !u256_eq(F::canon(F::mul(aff[k].x, z2)), F::canon(iso[k].x));
    bad += !u256_eq(F::canon(F::mul(aff[k].y, z3)), F::canon(iso[k].y));
  }
  return bad;
}

