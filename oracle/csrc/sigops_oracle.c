/*
 * sigops_oracle.c -- CPU oracle of the batch signature path (TEST
 * INFRASTRUCTURE ONLY: used by tests/, smoke() and bench.py's CPU-baseline
 * leg; never linked into libsigops.so).
 *
 * Plain-C restatement of what oracle/sigops_oracle.py states in Python
 * integers, for sizes the Python oracle cannot finish in seconds:
 *   - secp256k1 / P-256 ECDSA public-key recovery with fuel-crypto's 64-byte
 *     encoding and libsecp256k1 / p256 validity rules (the reference's
 *     arkworks_recover, src/curve_algos/secp256k1_ecdsa.rs:66-120, and the
 *     WGSL path src/wgsl/secp256k1_ecdsa.wgsl:87-130);
 *   - ed25519 verification with ed25519-dalek 2.1.1 semantics
 *     (src/curve_algos/ed25519_eddsa.rs:49-184);
 *   - signing helpers used to build test inputs (RFC 8032 for ed25519, ECDSA
 *     with a caller-given nonce, low-s, parity bit in s[0] bit 7).
 * Arithmetic: 4 x 64-bit limbs, Montgomery multiplication (CIOS) with
 * unsigned __int128, Fermat inversion, Jacobian / extended coordinates,
 * width-5 wNAF Strauss-Shamir.  Portable C (no intrinsics), same results on
 * x86-64 and aarch64.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;
typedef struct { uint64_t v[4]; } fe;

typedef struct {
  fe p, r2, one; /* modulus, R^2 mod p, R mod p (R = 2^256) */
  uint64_t ninv; /* -p^-1 mod 2^64 */
} mod_t;

enum { ST_OK = 0, ST_BAD_SCALAR = 1, ST_NO_POINT = 2, ST_INFINITY = 3, ST_MISMATCH = 4 };

/* ---------------------------------------------------------------- bigint */
static int fe_cmp(const fe *a, const fe *b) {
  for (int i = 3; i >= 0; --i) {
    if (a->v[i] < b->v[i]) return -1;
    if (a->v[i] > b->v[i]) return 1;
  }
  return 0;
}
static int fe_is_zero(const fe *a) { return (a->v[0] | a->v[1] | a->v[2] | a->v[3]) == 0; }
static uint64_t fe_add_raw(fe *r, const fe *a, const fe *b) {
  u128 c = 0;
  for (int i = 0; i < 4; ++i) { c += (u128)a->v[i] + b->v[i]; r->v[i] = (uint64_t)c; c >>= 64; }
  return (uint64_t)c;
}
static uint64_t fe_sub_raw(fe *r, const fe *a, const fe *b) {
  uint64_t br = 0;
  for (int i = 0; i < 4; ++i) {
    u128 d = (u128)a->v[i] - b->v[i] - br;
    r->v[i] = (uint64_t)d;
    br = (uint64_t)(d >> 64) & 1;
  }
  return br;
}
static void fe_from_be(fe *r, const uint8_t *b) {
  for (int i = 0; i < 4; ++i) {
    uint64_t w = 0;
    for (int k = 0; k < 8; ++k) w = (w << 8) | b[(3 - i) * 8 + k];
    r->v[i] = w;
  }
}
static void fe_to_be(uint8_t *b, const fe *a) {
  for (int i = 0; i < 4; ++i)
    for (int k = 0; k < 8; ++k) b[(3 - i) * 8 + k] = (uint8_t)(a->v[i] >> (56 - 8 * k));
}
static void fe_from_le(fe *r, const uint8_t *b) {
  for (int i = 0; i < 4; ++i) {
    uint64_t w = 0;
    for (int k = 7; k >= 0; --k) w = (w << 8) | b[i * 8 + k];
    r->v[i] = w;
  }
}
static void fe_to_le(uint8_t *b, const fe *a) {
  for (int i = 0; i < 4; ++i)
    for (int k = 0; k < 8; ++k) b[i * 8 + k] = (uint8_t)(a->v[i] >> (8 * k));
}
static void fe_set_u64(fe *r, uint64_t x) { r->v[0] = x; r->v[1] = r->v[2] = r->v[3] = 0; }

/* ---------------------------------------------------------- modular ops */
static void m_add(fe *r, const fe *a, const fe *b, const mod_t *m) {
  fe t, u;
  uint64_t c = fe_add_raw(&t, a, b);
  uint64_t br = fe_sub_raw(&u, &t, &m->p);
  *r = (c || !br) ? u : t;
}
static void m_sub(fe *r, const fe *a, const fe *b, const mod_t *m) {
  fe t;
  if (fe_sub_raw(&t, a, b)) fe_add_raw(&t, &t, &m->p);
  *r = t;
}
static void m_neg(fe *r, const fe *a, const mod_t *m) {
  if (fe_is_zero(a)) { *r = *a; return; }
  fe_sub_raw(r, &m->p, a);
}
static void m_mul(fe *r, const fe *a, const fe *b, const mod_t *m) {
  uint64_t t[6] = {0, 0, 0, 0, 0, 0};
  for (int i = 0; i < 4; ++i) {
    u128 s;
    uint64_t C = 0;
    for (int j = 0; j < 4; ++j) {
      s = (u128)a->v[j] * b->v[i] + t[j] + C;
      t[j] = (uint64_t)s;
      C = (uint64_t)(s >> 64);
    }
    s = (u128)t[4] + C;
    t[4] = (uint64_t)s;
    t[5] = (uint64_t)(s >> 64);
    uint64_t q = t[0] * m->ninv;
    s = (u128)q * m->p.v[0] + t[0];
    C = (uint64_t)(s >> 64);
    for (int j = 1; j < 4; ++j) {
      s = (u128)q * m->p.v[j] + t[j] + C;
      t[j - 1] = (uint64_t)s;
      C = (uint64_t)(s >> 64);
    }
    s = (u128)t[4] + C;
    t[3] = (uint64_t)s;
    t[4] = t[5] + (uint64_t)(s >> 64);
  }
  fe res = {{t[0], t[1], t[2], t[3]}}, u;
  uint64_t br = fe_sub_raw(&u, &res, &m->p);
  *r = (t[4] || !br) ? u : res;
}
static void m_sqr(fe *r, const fe *a, const mod_t *m) { m_mul(r, a, a, m); }
static void m_to(fe *r, const fe *a, const mod_t *m) { m_mul(r, a, &m->r2, m); }   /* any a < 2^256 */
static void m_from(fe *r, const fe *a, const mod_t *m) { fe one; fe_set_u64(&one, 1); m_mul(r, a, &one, m); }
static void m_pow(fe *r, const fe *a, const fe *e, const mod_t *m) { /* Montgomery domain */
  fe acc = m->one;
  for (int i = 255; i >= 0; --i) {
    m_sqr(&acc, &acc, m);
    if ((e->v[i >> 6] >> (i & 63)) & 1) m_mul(&acc, &acc, a, m);
  }
  *r = acc;
}
static void m_inv(fe *r, const fe *a, const mod_t *m) {
  fe e, two;
  fe_set_u64(&two, 2);
  fe_sub_raw(&e, &m->p, &two);
  m_pow(r, a, &e, m);
}
static int m_eq(const fe *a, const fe *b) { return fe_cmp(a, b) == 0; }

static void mod_init(mod_t *m, const uint64_t p[4]) {
  for (int i = 0; i < 4; ++i) m->p.v[i] = p[i];
  uint64_t inv = 1; /* Newton: p^-1 mod 2^64 */
  for (int i = 0; i < 7; ++i) inv *= 2 - p[0] * inv;
  m->ninv = (uint64_t)0 - inv;
  fe x;
  fe_set_u64(&x, 1);
  for (int i = 0; i < 512; ++i) {
    m_add(&x, &x, &x, m);
    if (i == 255) m->one = x;
  }
  m->r2 = x;
}

/* ------------------------------------------------------------- curves */
typedef struct { fe X, Y, Z; } jac; /* Z == 0: infinity */
typedef struct {
  mod_t fp, fn;
  fe a, b;     /* Montgomery form */
  fe gx, gy;   /* Montgomery form */
  int a_is_zero;
} wcurve;

static wcurve K1, R1;
static mod_t EDP, EDL;
static fe ED_D, ED_D2, ED_SQRTM1, ED_BX, ED_BY; /* Montgomery form (EDP) */
static pthread_once_t g_once = PTHREAD_ONCE_INIT;

static void hexfe(fe *r, const char *hex) {
  uint8_t b[32];
  for (int i = 0; i < 32; ++i) {
    int hi = hex[2 * i], lo = hex[2 * i + 1];
    hi = hi <= '9' ? hi - '0' : (hi | 32) - 'a' + 10;
    lo = lo <= '9' ? lo - '0' : (lo | 32) - 'a' + 10;
    b[i] = (uint8_t)(hi * 16 + lo);
  }
  fe_from_be(r, b);
}

static void jac_dbl(const wcurve *c, jac *r, const jac *p) {
  const mod_t *m = &c->fp;
  if (fe_is_zero(&p->Z) || fe_is_zero(&p->Y)) { memset(r, 0, sizeof *r); return; }
  fe YY, S, ZZ, M, t, X3, Y3, Z3;
  m_sqr(&YY, &p->Y, m);
  m_mul(&S, &p->X, &YY, m);
  m_add(&S, &S, &S, m); m_add(&S, &S, &S, m);
  m_sqr(&ZZ, &p->Z, m);
  m_sqr(&M, &p->X, m);
  m_add(&t, &M, &M, m); m_add(&M, &t, &M, m);
  if (!c->a_is_zero) { m_sqr(&t, &ZZ, m); m_mul(&t, &t, &c->a, m); m_add(&M, &M, &t, m); }
  m_sqr(&X3, &M, m);
  m_sub(&X3, &X3, &S, m); m_sub(&X3, &X3, &S, m);
  m_sub(&t, &S, &X3, m);
  m_mul(&Y3, &M, &t, m);
  m_sqr(&t, &YY, m);
  m_add(&t, &t, &t, m); m_add(&t, &t, &t, m); m_add(&t, &t, &t, m);
  m_sub(&Y3, &Y3, &t, m);
  m_mul(&Z3, &p->Y, &p->Z, m);
  m_add(&Z3, &Z3, &Z3, m);
  r->X = X3; r->Y = Y3; r->Z = Z3;
}

static void jac_add(const wcurve *c, jac *r, const jac *p, const jac *q) {
  const mod_t *m = &c->fp;
  if (fe_is_zero(&p->Z)) { *r = *q; return; }
  if (fe_is_zero(&q->Z)) { *r = *p; return; }
  fe Z1Z1, Z2Z2, U1, U2, S1, S2, H, R, HH, HHH, V, t, X3, Y3, Z3;
  m_sqr(&Z1Z1, &p->Z, m);
  m_sqr(&Z2Z2, &q->Z, m);
  m_mul(&U1, &p->X, &Z2Z2, m);
  m_mul(&U2, &q->X, &Z1Z1, m);
  m_mul(&t, &q->Z, &Z2Z2, m); m_mul(&S1, &p->Y, &t, m);
  m_mul(&t, &p->Z, &Z1Z1, m); m_mul(&S2, &q->Y, &t, m);
  m_sub(&H, &U2, &U1, m);
  m_sub(&R, &S2, &S1, m);
  if (fe_is_zero(&H)) {
    if (fe_is_zero(&R)) { jac_dbl(c, r, p); return; }
    memset(r, 0, sizeof *r);
    return;
  }
  m_sqr(&HH, &H, m);
  m_mul(&HHH, &H, &HH, m);
  m_mul(&V, &U1, &HH, m);
  m_sqr(&X3, &R, m);
  m_sub(&X3, &X3, &HHH, m); m_sub(&X3, &X3, &V, m); m_sub(&X3, &X3, &V, m);
  m_sub(&t, &V, &X3, m); m_mul(&Y3, &R, &t, m);
  m_mul(&t, &S1, &HHH, m); m_sub(&Y3, &Y3, &t, m);
  m_mul(&Z3, &p->Z, &q->Z, m); m_mul(&Z3, &Z3, &H, m);
  r->X = X3; r->Y = Y3; r->Z = Z3;
}

static void jac_neg(const wcurve *c, jac *r, const jac *p) { *r = *p; m_neg(&r->Y, &p->Y, &c->fp); }

/* width-w NAF of k (< 2^256) into naf[0..257), returns length */
static int wnaf(int8_t *naf, const fe *k, int w) {
  fe x = *k;
  int len = 0;
  memset(naf, 0, 260);
  const int64_t half = 1 << (w - 1), full = 1 << w;
  uint64_t carry_top = 0;
  while (!fe_is_zero(&x) || carry_top) {
    int8_t d = 0;
    if (x.v[0] & 1) {
      int64_t v = (int64_t)(x.v[0] & (uint64_t)(full - 1));
      if (v >= half) v -= full;
      d = (int8_t)v;
      fe t;
      if (v > 0) { fe_set_u64(&t, (uint64_t)v); fe_sub_raw(&x, &x, &t); }
      else { fe_set_u64(&t, (uint64_t)(-v)); carry_top += fe_add_raw(&x, &x, &t); }
    }
    naf[len++] = d;
    /* x >>= 1, bringing in the carry bit at the top */
    for (int i = 0; i < 3; ++i) x.v[i] = (x.v[i] >> 1) | (x.v[i + 1] << 63);
    x.v[3] = (x.v[3] >> 1) | (carry_top << 63);
    carry_top = 0;
  }
  return len;
}

/* k1*P + k2*Q, wNAF-5 Strauss-Shamir; P, Q Jacobian (non-infinity) */
static void jac_lincomb(const wcurve *c, jac *r, const fe *k1, const jac *P, const fe *k2, const jac *Q) {
  jac tp[8], tq[8], p2, q2;
  tp[0] = *P; tq[0] = *Q;
  jac_dbl(c, &p2, P); jac_dbl(c, &q2, Q);
  for (int i = 1; i < 8; ++i) { jac_add(c, &tp[i], &tp[i - 1], &p2); jac_add(c, &tq[i], &tq[i - 1], &q2); }
  int8_t n1[260], n2[260];
  int l1 = wnaf(n1, k1, 5), l2 = wnaf(n2, k2, 5);
  int len = l1 > l2 ? l1 : l2;
  jac acc;
  memset(&acc, 0, sizeof acc);
  for (int i = len - 1; i >= 0; --i) {
    jac_dbl(c, &acc, &acc);
    jac e;
    if (n1[i]) {
      int d = n1[i];
      if (d > 0) e = tp[(d - 1) / 2]; else jac_neg(c, &e, &tp[(-d - 1) / 2]);
      jac_add(c, &acc, &acc, &e);
    }
    if (n2[i]) {
      int d = n2[i];
      if (d > 0) e = tq[(d - 1) / 2]; else jac_neg(c, &e, &tq[(-d - 1) / 2]);
      jac_add(c, &acc, &acc, &e);
    }
  }
  *r = acc;
}

static void jac_mul(const wcurve *c, jac *r, const fe *k, const jac *P) {
  fe zero = {{0, 0, 0, 0}};
  jac_lincomb(c, r, k, P, &zero, P);
}

static int ecdsa_recover(const wcurve *c, const uint8_t *sig, const uint8_t *msg, uint8_t *out) {
  memset(out, 0, 64);
  const mod_t *fp = &c->fp, *fn = &c->fn;
  fe r, s, z, x, rhs, y, t;
  uint8_t sb[32];
  memcpy(sb, sig + 32, 32);
  int parity = sb[0] >> 7;
  sb[0] &= 0x7f;
  fe_from_be(&r, sig);
  fe_from_be(&s, sb);
  fe_from_be(&z, msg);
  if (fe_cmp(&z, &fn->p) >= 0) fe_sub_raw(&z, &z, &fn->p);
  if (fe_is_zero(&r) || fe_cmp(&r, &fn->p) >= 0 || fe_is_zero(&s) || fe_cmp(&s, &fn->p) >= 0) return ST_BAD_SCALAR;
  m_to(&x, &r, fp);
  m_sqr(&rhs, &x, fp);
  m_add(&rhs, &rhs, &c->a, fp);
  m_mul(&rhs, &rhs, &x, fp);
  m_add(&rhs, &rhs, &c->b, fp);
  fe e, one;
  fe_set_u64(&one, 1);
  fe_add_raw(&e, &fp->p, &one);
  for (int i = 0; i < 2; ++i) /* e = (p + 1) / 4 */
    for (int k = 0; k < 4; ++k) e.v[k] = (e.v[k] >> 1) | (k < 3 ? e.v[k + 1] << 63 : 0);
  m_pow(&y, &rhs, &e, fp);
  m_sqr(&t, &y, fp);
  if (!m_eq(&t, &rhs)) return ST_NO_POINT;
  fe yi;
  m_from(&yi, &y, fp);
  if ((int)(yi.v[0] & 1) != parity) m_neg(&y, &y, fp);
  /* scalars: u1 = -z/r, u2 = s/r */
  fe rm, rinv, u1, u2, zm, sm;
  m_to(&rm, &r, fn);
  m_inv(&rinv, &rm, fn);
  m_to(&zm, &z, fn); m_mul(&u1, &zm, &rinv, fn); m_from(&u1, &u1, fn); m_neg(&u1, &u1, fn);
  m_to(&sm, &s, fn); m_mul(&u2, &sm, &rinv, fn); m_from(&u2, &u2, fn);
  jac G = {c->gx, c->gy, c->fp.one}, R = {x, y, c->fp.one}, Q;
  jac_lincomb(c, &Q, &u1, &G, &u2, &R);
  if (fe_is_zero(&Q.Z)) return ST_INFINITY;
  fe zi, zi2, ax, ay;
  m_inv(&zi, &Q.Z, fp);
  m_sqr(&zi2, &zi, fp);
  m_mul(&ax, &Q.X, &zi2, fp);
  m_mul(&zi2, &zi2, &zi, fp);
  m_mul(&ay, &Q.Y, &zi2, fp);
  m_from(&ax, &ax, fp);
  m_from(&ay, &ay, fp);
  fe_to_be(out, &ax);
  fe_to_be(out + 32, &ay);
  return ST_OK;
}

/* ------------------------------------------------------------- SHA-512 */
static const uint64_t SHA_K[80] = {
#include "sha512_k.inc"
};
static uint64_t rotr(uint64_t x, int n) { return (x >> n) | (x << (64 - n)); }
static void sha512_block(uint64_t h[8], const uint8_t *blk) {
  uint64_t w[80];
  for (int i = 0; i < 16; ++i) {
    uint64_t v = 0;
    for (int k = 0; k < 8; ++k) v = (v << 8) | blk[8 * i + k];
    w[i] = v;
  }
  for (int i = 16; i < 80; ++i) {
    uint64_t s0 = rotr(w[i - 15], 1) ^ rotr(w[i - 15], 8) ^ (w[i - 15] >> 7);
    uint64_t s1 = rotr(w[i - 2], 19) ^ rotr(w[i - 2], 61) ^ (w[i - 2] >> 6);
    w[i] = w[i - 16] + s0 + w[i - 7] + s1;
  }
  uint64_t a = h[0], b = h[1], c = h[2], d = h[3], e = h[4], f = h[5], g = h[6], hh = h[7];
  for (int i = 0; i < 80; ++i) {
    uint64_t t1 = hh + (rotr(e, 14) ^ rotr(e, 18) ^ rotr(e, 41)) + ((e & f) ^ (~e & g)) + SHA_K[i] + w[i];
    uint64_t t2 = (rotr(a, 28) ^ rotr(a, 34) ^ rotr(a, 39)) + ((a & b) ^ (a & c) ^ (b & c));
    hh = g; g = f; f = e; e = d + t1; d = c; c = b; b = a; a = t1 + t2;
  }
  h[0] += a; h[1] += b; h[2] += c; h[3] += d; h[4] += e; h[5] += f; h[6] += g; h[7] += hh;
}
void sigops_oracle_sha512(const uint8_t *msg, size_t len, uint8_t out[64]) {
  uint64_t h[8] = {
#include "sha512_h.inc"
  };
  size_t off = 0;
  for (; len - off >= 128; off += 128) sha512_block(h, msg + off);
  uint8_t blk[256];
  size_t rem = len - off;
  memset(blk, 0, sizeof blk);
  memcpy(blk, msg + off, rem);
  blk[rem] = 0x80;
  size_t nb = rem + 17 <= 128 ? 1 : 2;
  uint64_t bits = (uint64_t)len * 8;
  for (int k = 0; k < 8; ++k) blk[nb * 128 - 1 - k] = (uint8_t)(bits >> (8 * k));
  for (size_t i = 0; i < nb; ++i) sha512_block(h, blk + 128 * i);
  for (int i = 0; i < 8; ++i)
    for (int k = 0; k < 8; ++k) out[8 * i + k] = (uint8_t)(h[i] >> (56 - 8 * k));
}

/* ------------------------------------------------------------- ed25519 */
typedef struct { fe X, Y, Z, T; } ept;

static void ed_add(ept *r, const ept *p, const ept *q) { /* unified, complete */
  const mod_t *m = &EDP;
  fe A, B, C, D, E, F, G, H, t;
  m_sub(&A, &p->Y, &p->X, m); m_sub(&t, &q->Y, &q->X, m); m_mul(&A, &A, &t, m);
  m_add(&B, &p->Y, &p->X, m); m_add(&t, &q->Y, &q->X, m); m_mul(&B, &B, &t, m);
  m_mul(&C, &p->T, &q->T, m); m_mul(&C, &C, &ED_D2, m);
  m_mul(&D, &p->Z, &q->Z, m); m_add(&D, &D, &D, m);
  m_sub(&E, &B, &A, m); m_sub(&F, &D, &C, m); m_add(&G, &D, &C, m); m_add(&H, &B, &A, m);
  m_mul(&r->X, &E, &F, m); m_mul(&r->Y, &G, &H, m); m_mul(&r->T, &E, &H, m); m_mul(&r->Z, &F, &G, m);
}

static void ed_identity(ept *r) {
  memset(r, 0, sizeof *r);
  r->Y = EDP.one;
  r->Z = EDP.one;
}

static void ed_neg(ept *r, const ept *p) { *r = *p; m_neg(&r->X, &p->X, &EDP); m_neg(&r->T, &p->T, &EDP); }

static void ed_lincomb(ept *r, const fe *k1, const ept *P, const fe *k2, const ept *Q) {
  ept tp[8], tq[8], p2, q2;
  tp[0] = *P; tq[0] = *Q;
  ed_add(&p2, P, P); ed_add(&q2, Q, Q);
  for (int i = 1; i < 8; ++i) { ed_add(&tp[i], &tp[i - 1], &p2); ed_add(&tq[i], &tq[i - 1], &q2); }
  int8_t n1[260], n2[260];
  int l1 = wnaf(n1, k1, 5), l2 = wnaf(n2, k2, 5);
  int len = l1 > l2 ? l1 : l2;
  ept acc, e;
  ed_identity(&acc);
  for (int i = len - 1; i >= 0; --i) {
    ed_add(&acc, &acc, &acc);
    if (n1[i]) { int d = n1[i]; if (d > 0) e = tp[(d - 1) / 2]; else ed_neg(&e, &tp[(-d - 1) / 2]); ed_add(&acc, &acc, &e); }
    if (n2[i]) { int d = n2[i]; if (d > 0) e = tq[(d - 1) / 2]; else ed_neg(&e, &tq[(-d - 1) / 2]); ed_add(&acc, &acc, &e); }
  }
  *r = acc;
}

static void ed_compress(uint8_t out[32], const ept *p) {
  fe zi, x, y;
  m_inv(&zi, &p->Z, &EDP);
  m_mul(&x, &p->X, &zi, &EDP);
  m_mul(&y, &p->Y, &zi, &EDP);
  m_from(&x, &x, &EDP);
  m_from(&y, &y, &EDP);
  fe_to_le(out, &y);
  out[31] |= (uint8_t)((x.v[0] & 1) << 7);
}

/* curve25519-dalek sqrt_ratio_i (src/curve_algos/ed25519_eddsa.rs:160-184), Montgomery domain */
static int sqrt_ratio_i(fe *r_out, const fe *u, const fe *v) {
  const mod_t *m = &EDP;
  fe v3, v7, r, check, nu, nui, t, e, x5;
  m_sqr(&v3, v, m); m_mul(&v3, &v3, v, m);
  m_sqr(&v7, &v3, m); m_mul(&v7, &v7, v, m);
  fe_set_u64(&x5, 5);
  fe_sub_raw(&e, &m->p, &x5);
  for (int i = 0; i < 3; ++i) /* (p - 5) / 8 */
    for (int k = 0; k < 4; ++k) e.v[k] = (e.v[k] >> 1) | (k < 3 ? e.v[k + 1] << 63 : 0);
  m_mul(&t, u, &v7, m);
  m_pow(&t, &t, &e, m);
  m_mul(&r, u, &v3, m);
  m_mul(&r, &r, &t, m);
  m_sqr(&check, &r, m); m_mul(&check, &check, v, m);
  m_neg(&nu, u, m);
  m_mul(&nui, &nu, &ED_SQRTM1, m);
  int correct = m_eq(&check, u), flipped = m_eq(&check, &nu), flipped_i = m_eq(&check, &nui);
  if (flipped || flipped_i) m_mul(&r, &r, &ED_SQRTM1, m);
  fe ri;
  m_from(&ri, &r, m);
  if (ri.v[0] & 1) m_neg(&r, &r, m);
  *r_out = r;
  return correct || flipped;
}

/* dalek CompressedEdwardsY::decompress: y mod p from the low 255 bits */
static int ed_decompress(ept *out, const uint8_t enc[32]) {
  const mod_t *m = &EDP;
  uint8_t b[32];
  memcpy(b, enc, 32);
  int sign = b[31] >> 7;
  b[31] &= 0x7f;
  fe y, yy, u, v, x;
  fe_from_le(&y, b);
  if (fe_cmp(&y, &m->p) >= 0) fe_sub_raw(&y, &y, &m->p);
  m_to(&y, &y, m);
  m_sqr(&yy, &y, m);
  m_sub(&u, &yy, &m->one, m);
  m_mul(&v, &yy, &ED_D, m);
  m_add(&v, &v, &m->one, m);
  if (!sqrt_ratio_i(&x, &u, &v)) return 0;
  if (sign) m_neg(&x, &x, m);
  out->X = x; out->Y = y; out->Z = m->one;
  m_mul(&out->T, &x, &y, m);
  return 1;
}

/* 64-byte little-endian hash mod l */
static void reduce512_mod_l(fe *k, const uint8_t h[64]) {
  fe lo, hi, t, R2 = EDL.r2;
  fe_from_le(&lo, h);
  fe_from_le(&hi, h + 32);
  m_to(&lo, &lo, &EDL);                 /* lo * R */
  m_to(&hi, &hi, &EDL);                 /* hi * R */
  m_mul(&hi, &hi, &R2, &EDL);           /* hi * R * R = (hi * 2^256) * R */
  m_add(&t, &lo, &hi, &EDL);
  m_from(k, &t, &EDL);
}

static int ed_verify(const uint8_t *sig, const uint8_t *msg, const uint8_t *pk) {
  ept A, negA, B, Rp;
  if (!ed_decompress(&A, pk)) return ST_NO_POINT;
  fe S;
  fe_from_le(&S, sig + 32);
  if (fe_cmp(&S, &EDL.p) >= 0) return ST_BAD_SCALAR;
  uint8_t pre[96], h[64], enc[32];
  memcpy(pre, sig, 32); memcpy(pre + 32, pk, 32); memcpy(pre + 64, msg, 32);
  sigops_oracle_sha512(pre, 96, h);
  fe k;
  reduce512_mod_l(&k, h);
  ed_neg(&negA, &A);
  B.X = ED_BX; B.Y = ED_BY; B.Z = EDP.one;
  m_mul(&B.T, &ED_BX, &ED_BY, &EDP);
  ed_lincomb(&Rp, &S, &B, &k, &negA);
  ed_compress(enc, &Rp);
  return memcmp(enc, sig, 32) == 0 ? ST_OK : ST_MISMATCH;
}

/* ---------------------------------------------------------------- init */
static void init_consts(void) {
  static const uint64_t k1p[4] = {0xFFFFFFFEFFFFFC2Full, ~0ull, ~0ull, ~0ull};
  static const uint64_t k1n[4] = {0xBFD25E8CD0364141ull, 0xBAAEDCE6AF48A03Bull, 0xFFFFFFFFFFFFFFFEull, ~0ull};
  static const uint64_t r1p[4] = {~0ull, 0x00000000FFFFFFFFull, 0ull, 0xFFFFFFFF00000001ull};
  static const uint64_t r1n[4] = {0xF3B9CAC2FC632551ull, 0xBCE6FAADA7179E84ull, ~0ull, 0xFFFFFFFF00000000ull};
  static const uint64_t edp[4] = {0xFFFFFFFFFFFFFFEDull, ~0ull, ~0ull, 0x7FFFFFFFFFFFFFFFull};
  static const uint64_t edl[4] = {0x5812631A5CF5D3EDull, 0x14DEF9DEA2F79CD6ull, 0ull, 0x1000000000000000ull};
  fe t;
  mod_init(&K1.fp, k1p); mod_init(&K1.fn, k1n);
  memset(&K1.a, 0, sizeof(fe));
  K1.a_is_zero = 1;
  fe_set_u64(&t, 7); m_to(&K1.b, &t, &K1.fp);
  hexfe(&t, "79BE667EF9DCBBAC55A06295CE870B07029BFCDB2DCE28D959F2815B16F81798"); m_to(&K1.gx, &t, &K1.fp);
  hexfe(&t, "483ADA7726A3C4655DA4FBFC0E1108A8FD17B448A68554199C47D08FFB10D4B8"); m_to(&K1.gy, &t, &K1.fp);
  mod_init(&R1.fp, r1p); mod_init(&R1.fn, r1n);
  fe_set_u64(&t, 3); m_to(&t, &t, &R1.fp); m_neg(&R1.a, &t, &R1.fp);
  R1.a_is_zero = 0;
  hexfe(&t, "5AC635D8AA3A93E7B3EBBD55769886BC651D06B0CC53B0F63BCE3C3E27D2604B"); m_to(&R1.b, &t, &R1.fp);
  hexfe(&t, "6B17D1F2E12C4247F8BCE6E563A440F277037D812DEB33A0F4A13945D898C296"); m_to(&R1.gx, &t, &R1.fp);
  hexfe(&t, "4FE342E2FE1A7F9B8EE7EB4A7C0F9E162BCE33576B315ECECBB6406837BF51F5"); m_to(&R1.gy, &t, &R1.fp);
  mod_init(&EDP, edp); mod_init(&EDL, edl);
  /* d = -121665 / 121666 */
  fe n1, d1;
  fe_set_u64(&n1, 121665); m_to(&n1, &n1, &EDP); m_neg(&n1, &n1, &EDP);
  fe_set_u64(&d1, 121666); m_to(&d1, &d1, &EDP); m_inv(&d1, &d1, &EDP);
  m_mul(&ED_D, &n1, &d1, &EDP);
  m_add(&ED_D2, &ED_D, &ED_D, &EDP);
  /* sqrt(-1) = 2^((p-1)/4) */
  fe two, e;
  fe_set_u64(&two, 2); m_to(&two, &two, &EDP);
  fe_set_u64(&t, 1); fe_sub_raw(&e, &EDP.p, &t);
  for (int i = 0; i < 2; ++i)
    for (int k = 0; k < 4; ++k) e.v[k] = (e.v[k] >> 1) | (k < 3 ? e.v[k + 1] << 63 : 0);
  m_pow(&ED_SQRTM1, &two, &e, &EDP);
  /* base point: y = 4/5, x even */
  fe four, five;
  fe_set_u64(&four, 4); m_to(&four, &four, &EDP);
  fe_set_u64(&five, 5); m_to(&five, &five, &EDP); m_inv(&five, &five, &EDP);
  m_mul(&ED_BY, &four, &five, &EDP);
  uint8_t enc[32];
  fe yi;
  m_from(&yi, &ED_BY, &EDP);
  fe_to_le(enc, &yi);
  ept b;
  ed_decompress(&b, enc);
  ED_BX = b.X;
}
static void ensure_init(void) { pthread_once(&g_once, init_consts); }

/* --------------------------------------------------------- public API */
int sigops_oracle_secp256k1_recover(const uint8_t *sig, const uint8_t *msg, uint8_t *out) { ensure_init(); return ecdsa_recover(&K1, sig, msg, out); }
int sigops_oracle_secp256r1_recover(const uint8_t *sig, const uint8_t *msg, uint8_t *out) { ensure_init(); return ecdsa_recover(&R1, sig, msg, out); }
int sigops_oracle_ed25519_verify(const uint8_t *sig, const uint8_t *msg, const uint8_t *pk) { ensure_init(); return ed_verify(sig, msg, pk); }

/* ECDSA signature with nonce k (32 bytes BE, 0 < k < n) and secret d; fuel
 * encoding.  Returns 0, or -1 if k or d is unusable (r = 0, s = 0, R.x >= n). */
int sigops_oracle_ecdsa_sign(int curve, const uint8_t *d32, const uint8_t *msg, const uint8_t *k32, uint8_t *sig, uint8_t *pub) {
  ensure_init();
  const wcurve *c = curve == 0 ? &K1 : &R1;
  const mod_t *fp = &c->fp, *fn = &c->fn;
  fe d, k, z;
  fe_from_be(&d, d32);
  fe_from_be(&k, k32);
  fe_from_be(&z, msg);
  if (fe_cmp(&z, &fn->p) >= 0) fe_sub_raw(&z, &z, &fn->p);
  if (fe_is_zero(&k) || fe_cmp(&k, &fn->p) >= 0 || fe_is_zero(&d) || fe_cmp(&d, &fn->p) >= 0) return -1;
  jac G = {c->gx, c->gy, c->fp.one}, R, Q;
  jac_mul(c, &R, &k, &G);
  fe zi, zi2, rx, ry;
  m_inv(&zi, &R.Z, fp); m_sqr(&zi2, &zi, fp);
  m_mul(&rx, &R.X, &zi2, fp); m_mul(&zi2, &zi2, &zi, fp); m_mul(&ry, &R.Y, &zi2, fp);
  m_from(&rx, &rx, fp); m_from(&ry, &ry, fp);
  if (fe_cmp(&rx, &fn->p) >= 0 || fe_is_zero(&rx)) return -1;
  int odd = (int)(ry.v[0] & 1);
  fe km, kinv, rm, dm, zm, s;
  m_to(&km, &k, fn); m_inv(&kinv, &km, fn);
  m_to(&rm, &rx, fn); m_to(&dm, &d, fn); m_to(&zm, &z, fn);
  m_mul(&s, &rm, &dm, fn); m_add(&s, &s, &zm, fn); m_mul(&s, &s, &kinv, fn); m_from(&s, &s, fn);
  if (fe_is_zero(&s)) return -1;
  fe half = fn->p;
  for (int k2 = 0; k2 < 4; ++k2) half.v[k2] = (half.v[k2] >> 1) | (k2 < 3 ? half.v[k2 + 1] << 63 : 0);
  if (fe_cmp(&s, &half) > 0) { fe_sub_raw(&s, &fn->p, &s); odd ^= 1; }
  fe_to_be(sig, &rx);
  fe_to_be(sig + 32, &s);
  sig[32] |= (uint8_t)(odd << 7);
  if (pub) {
    jac_mul(c, &Q, &d, &G);
    m_inv(&zi, &Q.Z, fp); m_sqr(&zi2, &zi, fp);
    m_mul(&rx, &Q.X, &zi2, fp); m_mul(&zi2, &zi2, &zi, fp); m_mul(&ry, &Q.Y, &zi2, fp);
    m_from(&rx, &rx, fp); m_from(&ry, &ry, fp);
    fe_to_be(pub, &rx); fe_to_be(pub + 32, &ry);
  }
  return 0;
}

/* RFC 8032 Ed25519 signing of a 32-byte message; also returns the key */
int sigops_oracle_ed25519_sign(const uint8_t *seed, const uint8_t *msg, uint8_t *sig, uint8_t *pk) {
  ensure_init();
  uint8_t h[64], buf[64], rh[64], pre[96];
  sigops_oracle_sha512(seed, 32, h);
  h[0] &= 248; h[31] &= 127; h[31] |= 64;
  fe a, r, k, S, t;
  fe_from_le(&a, h);
  ept B, A, R, id;
  B.X = ED_BX; B.Y = ED_BY; B.Z = EDP.one; m_mul(&B.T, &ED_BX, &ED_BY, &EDP);
  ed_identity(&id);
  fe zero = {{0, 0, 0, 0}};
  ed_lincomb(&A, &a, &B, &zero, &id);
  ed_compress(pk, &A);
  memcpy(buf, h + 32, 32); memcpy(buf + 32, msg, 32);
  sigops_oracle_sha512(buf, 64, rh);
  reduce512_mod_l(&r, rh);
  ed_lincomb(&R, &r, &B, &zero, &id);
  ed_compress(sig, &R);
  memcpy(pre, sig, 32); memcpy(pre + 32, pk, 32); memcpy(pre + 64, msg, 32);
  sigops_oracle_sha512(pre, 96, rh);
  reduce512_mod_l(&k, rh);
  /* S = r + k * a mod l (a < 2^255 reduced first) */
  fe am, km, rm;
  m_to(&am, &a, &EDL); m_to(&km, &k, &EDL); m_to(&rm, &r, &EDL);
  m_mul(&t, &km, &am, &EDL); m_add(&t, &t, &rm, &EDL); m_from(&S, &t, &EDL);
  fe_to_le(sig + 32, &S);
  return 0;
}

/* ---------------------------------------------------------- batch API */
typedef struct {
  int curve;
  const uint8_t *sigs, *msgs, *pks;
  uint8_t *out, *status;
  size_t lo, hi;
} job_t;

static void *worker(void *arg) {
  job_t *j = (job_t *)arg;
  for (size_t i = j->lo; i < j->hi; ++i) {
    int st;
    if (j->curve == 2) {
      st = ed_verify(j->sigs + 64 * i, j->msgs + 32 * i, j->pks + 32 * i);
      if (j->out) j->out[i] = st == ST_OK;
    } else {
      uint8_t tmp[64];
      st = ecdsa_recover(j->curve == 0 ? &K1 : &R1, j->sigs + 64 * i, j->msgs + 32 * i, tmp);
      if (j->out) memcpy(j->out + 64 * i, tmp, 64);
    }
    if (j->status) j->status[i] = (uint8_t)st;
  }
  return NULL;
}

/* curve 0/1: out n*64 keys; curve 2: out n validity bytes.  threads <= 0: 1 */
int sigops_oracle_batch(int curve, const uint8_t *sigs, const uint8_t *msgs, const uint8_t *pks, size_t n, uint8_t *out, uint8_t *status,
                        int threads) {
  ensure_init();
  if (curve < 0 || curve > 2) return -22;
  if (threads <= 1 || n < 2) {
    job_t j = {curve, sigs, msgs, pks, out, status, 0, n};
    worker(&j);
    return 0;
  }
  if ((size_t)threads > n) threads = (int)n;
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
  job_t *jobs = (job_t *)malloc(sizeof(job_t) * threads);
  for (int t = 0; t < threads; ++t) {
    jobs[t] = (job_t){curve, sigs, msgs, pks, out, status, n * t / threads, n * (t + 1) / threads};
    pthread_create(&th[t], NULL, worker, &jobs[t]);
  }
  for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
  free(th);
  free(jobs);
  return 0;
}

/* mixed batch: curve tag per item (0/1/2); out 64 bytes per item (key, or
 * validity in byte 0 for ed25519) */
typedef struct {
  const uint8_t *curves, *sigs, *msgs, *pks;
  uint8_t *out, *status;
  size_t lo, hi;
} mjob_t;

static void *mworker(void *arg) {
  mjob_t *j = (mjob_t *)arg;
  for (size_t i = j->lo; i < j->hi; ++i) {
    int st;
    uint8_t tmp[64];
    memset(tmp, 0, 64);
    if (j->curves[i] == 2) {
      st = ed_verify(j->sigs + 64 * i, j->msgs + 32 * i, j->pks + 32 * i);
      tmp[0] = st == ST_OK;
    } else {
      st = ecdsa_recover(j->curves[i] == 0 ? &K1 : &R1, j->sigs + 64 * i, j->msgs + 32 * i, tmp);
    }
    if (j->out) memcpy(j->out + 64 * i, tmp, 64);
    if (j->status) j->status[i] = (uint8_t)st;
  }
  return NULL;
}

int sigops_oracle_batch_mixed(const uint8_t *curves, const uint8_t *sigs, const uint8_t *msgs, const uint8_t *pks, size_t n, uint8_t *out,
                              uint8_t *status, int threads) {
  ensure_init();
  if (threads < 1) threads = 1;
  if ((size_t)threads > n) threads = n ? (int)n : 1;
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
  mjob_t *jobs = (mjob_t *)malloc(sizeof(mjob_t) * threads);
  for (int t = 0; t < threads; ++t) {
    jobs[t] = (mjob_t){curves, sigs, msgs, pks, out, status, n * t / threads, n * (t + 1) / threads};
    pthread_create(&th[t], NULL, mworker, &jobs[t]);
  }
  for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
  free(th);
  free(jobs);
  return 0;
}
