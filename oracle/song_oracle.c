/*
 * song_oracle.c -- CPU oracle for the batched best-first graph search.
 *
 * TEST INFRASTRUCTURE ONLY (see song_oracle.h).  Plain C11, no intrinsics, no
 * inline assembly; compiled with -ffp-contract=off so that every fused
 * multiply-add below is an explicit fmaf() and nothing else is contracted.
 * Builds and gives the same results on x86-64 and aarch64.
 */
#include "song_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* Distances                                                                 */
/* ------------------------------------------------------------------------- */

/* warp_astar_accelerator.h:115-163 (start vertex) and :237-287 (neighbours):
 * lane l accumulates dims l, l+32, ... in order; the 32 partial sums are
 * combined by tmp += shfl_xor(tmp, o) for o = 16, 8, 4, 2, 1, after which all
 * lanes hold the same value.  Cosine: sign * tmp * tmp / |x|^2 in float with
 * sign = (tmp < 0 ? 1 : -1), 0 when |x|^2 == 0; the query norm is not used. */
float orc_kernel_distance(int metric, int dim, const float *q, const float *x, int use_fma) {
  if (metric == ORC_HAMMING) {
    /* hash_warp_no_heap_astar_accelerator.h:96-104: __popc of the xor of the
     * code words, summed (an integer, exact as float); dim = code words */
    uint32_t qa, xa;
    int h = 0;
    for (int j = 0; j < dim; ++j) {
      memcpy(&qa, q + j, 4);
      memcpy(&xa, x + j, 4);
      h += __builtin_popcount(qa ^ xa);
    }
    return (float)h;
  }
  float t[32], l[32], nt[32], nl[32];
  for (int lane = 0; lane < 32; ++lane) {
    float a = 0.0f, b = 0.0f;
    for (int j = lane; j < dim; j += 32) {
      if (metric == ORC_L2) {
        float d = q[j] - x[j];
        if (use_fma) a = fmaf(d, d, a);
        else { float p = d * d; a = a + p; }
      } else {
        if (use_fma) a = fmaf(q[j], x[j], a);
        else { float p = q[j] * x[j]; a = a + p; }
        if (metric == ORC_COS) {
          if (use_fma) b = fmaf(x[j], x[j], b);
          else { float p = x[j] * x[j]; b = b + p; }
        }
      }
    }
    t[lane] = a;
    l[lane] = b;
  }
  for (int off = 16; off > 0; off >>= 1) {
    for (int lane = 0; lane < 32; ++lane) {
      nt[lane] = t[lane] + t[lane ^ off];
      nl[lane] = l[lane] + l[lane ^ off];
    }
    memcpy(t, nt, sizeof t);
    memcpy(l, nl, sizeof l);
  }
  if (metric == ORC_L2) return t[0];
  if (metric == ORC_IP) return -t[0];
  if (l[0] != 0.0f) {
    float sign = t[0] < 0.0f ? 1.0f : -1.0f;
    float st = sign * t[0];
    float num = st * t[0];
    return num / l[0];
  }
  return 0.0f;
}

/* data.h:28-62: float products accumulated in double; cosine keeps the two
 * squared norms in float and divides by both (x = base row, q = query). */
double orc_cpu_distance(int metric, int dim, const float *x, const float *q) {
  double ret = 0.0;
  if (metric == ORC_L2) {
    for (int i = 0; i < dim; ++i) {
      float diff = x[i] - q[i];
      float sq = diff * diff;
      ret += (double)sq;
    }
    return ret;
  }
  if (metric == ORC_IP) {
    for (int i = 0; i < dim; ++i) {
      float p = x[i] * q[i];
      ret -= (double)p;
    }
    return ret;
  }
  float lena = 0.0f, lenv = 0.0f;
  for (int i = 0; i < dim; ++i) {
    float p = x[i] * q[i];
    ret += (double)p;
    float pa = x[i] * x[i];
    lena = lena + pa;
    float pv = q[i] * q[i];
    lenv = lenv + pv;
  }
  int sign = ret < 0 ? 1 : -1;
  return (double)sign * (ret * ret / (double)lena / (double)lenv);
}

/* ------------------------------------------------------------------------- */
/* Visited hash: fixhash.h:3-109 with __ENABLE_VISITED_DEL                   */
/* ------------------------------------------------------------------------- */

#define FH_EMPTY (-1)
#define FH_DELETION (-2)
static const uint64_t FH_R0 = 0x4bcb391f924ed183ULL; /* fixhash.h:9, first multiplier */
static const uint64_t FH_R1 = 0xa0ab69ccd854fc0aULL; /* fixhash.h:9, first xor mask   */

/* hash(0, x) = (x ^ (x >> 16) * r0 ^ r1) % cap on 64-bit x, returned as short
 * (fixhash.h:20-24).  cap <= 32767 keeps the short cast exact. */
int orc_fixhash_hash(int cap, uint64_t x) {
  uint64_t v = x ^ ((x >> 16) * FH_R0) ^ FH_R1;
  return (int)(short)(v % (uint64_t)cap);
}

static inline int fh_home(int cap, int32_t x) {
  /* The table stores int; hash() receives it widened to idx_t (size_t). */
  return orc_fixhash_hash(cap, (uint64_t)(int64_t)x);
}

void orc_fixhash_init(int32_t *tab, int cap) {
  for (int i = 0; i < cap; ++i) tab[i] = FH_EMPTY;
}

/* fixhash.h:38-47: first EMPTY (or DELETION) slot on the probe sequence. */
void orc_fixhash_add(int32_t *tab, int cap, int32_t x) {
  int code = fh_home(cap, x);
  while (tab[code] != FH_EMPTY && tab[code] != FH_DELETION) code = (code + 1) % cap;
  tab[code] = x;
}

/* fixhash.h:49-57 */
int orc_fixhash_test(const int32_t *tab, int cap, int32_t x) {
  int code = fh_home(cap, x);
  while (tab[code] != FH_EMPTY) {
    if (tab[code] == x) return 1;
    code = (code + 1) % cap;
  }
  return 0;
}

/* fixhash.h:59-93: find x, then walk the run after it and pull entries back
 * into the hole under the reference's three position cases.  The cases test
 * the home of the entry that was moved last ("code"), not the hole, which is
 * why the table can lose an entry (a false negative in later tests); this
 * restatement keeps that behaviour. */
void orc_fixhash_del(int32_t *tab, int cap, int32_t x) {
  int code = fh_home(cap, x);
  int remove_idx = code;
  while (tab[remove_idx] != FH_EMPTY) {
    if (tab[remove_idx] == x) break;
    remove_idx = (remove_idx + 1) % cap;
  }
  if (tab[remove_idx] == FH_EMPTY) return;
  int next_idx = (remove_idx + 1) % cap;
  while (tab[next_idx] != FH_EMPTY) {
    int new_code = fh_home(cap, tab[next_idx]);
    int cond1 = code <= remove_idx;
    int cond2 = remove_idx < next_idx;
    int move;
    if (cond1 && cond2) move = new_code <= remove_idx;
    else if (cond1) move = next_idx < new_code && new_code <= remove_idx;
    else move = next_idx < new_code || new_code <= remove_idx;
    if (move) {
      tab[remove_idx] = tab[next_idx];
      remove_idx = next_idx;
      code = new_code;
    }
    next_idx = (next_idx + 1) % cap;
  }
  tab[remove_idx] = FH_EMPTY;
}

/* ------------------------------------------------------------------------- */
/* Reference queues: SMMH (smmh2.h) and binary max-heap (bin_heap.h)          */
/* Elements compare on the distance only (KernelPair, astar_accelerator.h).   */
/* ------------------------------------------------------------------------- */

typedef struct {
  double d;
  uint64_t id;
} kp_t;

static inline void kp_swap(kp_t *a, kp_t *b) {
  kp_t c = *a;
  *a = *b;
  *b = c;
}

/* smmh2.h:11-31 */
static int smmh_adjust_sibling(kp_t *h, int y, int hs) {
  if (y & 1) {
    int s = y + 1;
    if (s >= hs) return y;
    if (h[y].d > h[s].d) {
      kp_swap(&h[y], &h[s]);
      return s;
    }
  } else {
    int s = y - 1;
    if (h[y].d < h[s].d) {
      kp_swap(&h[y], &h[s]);
      return s;
    }
  }
  return y;
}

/* smmh2.h:58-73 */
static int smmh_adjust_grandparent(kp_t *h, int y) {
  if (y <= 2) return y;
  int g = (y - 3) >> 2;
  int gl = (g << 1) + 1, gr = (g << 1) + 2;
  if (h[gl].d > h[y].d) {
    kp_swap(&h[gl], &h[y]);
    return gl;
  } else if (h[gr].d < h[y].d) {
    kp_swap(&h[gr], &h[y]);
    return gr;
  }
  return y;
}

/* smmh2.h:75-88: slot 0 is unused, hs = live elements + 1 */
static void smmh_insert(kp_t *h, int *hs, kp_t e) {
  int y = *hs;
  h[(*hs)++] = e;
  for (;;) {
    y = smmh_adjust_sibling(h, y, *hs);
    int x = smmh_adjust_grandparent(h, y);
    if (x == y) break;
    y = x;
  }
}

/* smmh2.h:90-117 */
static int smmh_adjust_grandchild(kp_t *h, int y, int hs) {
  if (y & 1) {
    if ((y << 1) + 1 >= hs) return y;
    int cl = (y << 1) + 1, cr = ((y + 1) << 1) + 1;
    int c = cl;
    if (cr < hs && h[cr].d < h[cl].d) c = cr;
    if (h[c].d < h[y].d) {
      kp_swap(&h[c], &h[y]);
      return c;
    }
  } else {
    int cl = ((y - 1) << 1) + 2, cr = (y << 1) + 2;
    if (cl >= hs) return y;
    int c = cl;
    if (cr < hs && h[cr].d > h[cl].d) c = cr;
    if (h[c].d > h[y].d) {
      kp_swap(&h[c], &h[y]);
      return c;
    }
  }
  return y;
}

/* smmh2.h:119-131 (the sibling step's result is not used, as there) */
static void smmh_deletion(kp_t *h, int idx, int *hs) {
  h[idx] = h[--(*hs)];
  int y = idx;
  for (;;) {
    smmh_adjust_sibling(h, y, *hs);
    int x = smmh_adjust_grandchild(h, y, *hs);
    if (x == y) break;
    y = x;
  }
}

static kp_t smmh_pop_min(kp_t *h, int *hs) {
  kp_t r = h[1];
  smmh_deletion(h, 1, hs);
  return r;
}

static kp_t smmh_pop_max(kp_t *h, int *hs) {
  kp_t r = h[2];
  smmh_deletion(h, 2, hs);
  return r;
}

/* bin_heap.h:4-20 (C division truncates, so the root compares with itself) */
static void bh_push(kp_t *b, int len) {
  int now = len - 1;
  int parent = (now - 1) / 2;
  while (parent >= 0) {
    if (b[parent].d < b[now].d) {
      kp_swap(&b[parent], &b[now]);
      now = parent;
      parent = (parent - 1) / 2;
    } else {
      break;
    }
  }
}

/* bin_heap.h:21-47: the last slot stays inside the sift range */
static kp_t bh_pop(kp_t *b, int len) {
  kp_t ret = b[0];
  b[0] = b[len - 1];
  int now = 0;
  while (now + 1 < len) {
    int left = now * 2 + 1, right = now * 2 + 2, next = -1;
    if (right < len) next = b[left].d < b[right].d ? right : left;
    else if (left < len) next = left;
    if (next == -1 || !(b[now].d < b[next].d)) break;
    kp_swap(&b[now], &b[next]);
    now = next;
  }
  return ret;
}

/* ------------------------------------------------------------------------- */
/* Sorted queues of the GB300 kernel: key (distance, id), ascending           */
/* ------------------------------------------------------------------------- */

typedef struct {
  float d;
  uint32_t pad;
  uint64_t id;
} lk_t;

static inline int lk_less(lk_t a, lk_t b) { return a.d < b.d || (a.d == b.d && a.id < b.id); }

static void lk_insert(lk_t *a, int *n, lk_t e) {
  int pos = *n;
  while (pos > 0 && lk_less(e, a[pos - 1])) {
    a[pos] = a[pos - 1];
    --pos;
  }
  a[pos] = e;
  ++(*n);
}

/* ------------------------------------------------------------------------- */
/* Kernel-semantics search                                                    */
/* ------------------------------------------------------------------------- */

typedef struct {
  int pq;
  int maxdeg;
  uint16_t *cnt;      /* LEX_EXACT: visited multiplicity per vertex */
  uint64_t *touched;  /* LEX_EXACT: vertices with cnt != 0 to clear */
  size_t ntouched, tcap;
  kp_t *q, *t;   /* REF */
  lk_t *lq, *lt; /* LEX */
  int32_t *tab;
  uint64_t *cand;
  float *cdist;
  uint64_t *tmp_out;
} kscratch;

static int kscratch_init(kscratch *s, int pq, int maxdeg, uint64_t n) {
  memset(s, 0, sizeof *s);
  s->cnt = (uint16_t *)calloc((size_t)n, sizeof(uint16_t));
  s->pq = pq;
  s->maxdeg = maxdeg;
  s->q = (kp_t *)malloc(sizeof(kp_t) * (size_t)(pq + 3));
  s->t = (kp_t *)malloc(sizeof(kp_t) * (size_t)(pq + 2));
  s->lq = (lk_t *)malloc(sizeof(lk_t) * (size_t)(pq + 3));
  s->lt = (lk_t *)malloc(sizeof(lk_t) * (size_t)(pq + 2));
  s->tab = (int32_t *)malloc(sizeof(int32_t) * (size_t)8 * (size_t)pq);
  s->cand = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)ORC_MAX_PROBES * (size_t)(maxdeg + 1));
  s->cdist = (float *)malloc(sizeof(float) * (size_t)ORC_MAX_PROBES * (size_t)(maxdeg + 1));
  s->tmp_out = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)pq);
  return s->cnt && s->q && s->t && s->lq && s->lt && s->tab && s->cand && s->cdist && s->tmp_out ? 0 : -1;
}

static void kscratch_free(kscratch *s) {
  free(s->cnt);
  free(s->touched);
  free(s->q);
  free(s->t);
  free(s->lq);
  free(s->lt);
  free(s->tab);
  free(s->cand);
  free(s->cdist);
  free(s->tmp_out);
}

typedef struct {
  orc_event *log;
  int cap;
  int n;
} evlog;

static inline void ev(evlog *L, int kind, uint64_t id, float d) {
  if (!L) return;
  if (L->n < L->cap) {
    orc_event *e = &L->log[L->n];
    e->kind = kind;
    e->pad = 0;
    e->id = id;
    e->dist = d;
    e->pad2 = 0;
  }
  L->n++;
}

static inline const float *row(const orc_index *ix, uint64_t id) {
  return ix->data + id * (uint64_t)ix->dim;
}

/* Visited-set operations: FixHash (modes REF and LEX) or an exact multiset
 * (mode LEX_EXACT). */
typedef struct {
  int exact;
  int32_t *tab;
  int cap;
  kscratch *s;
} vset;

static void vs_add(vset *v, uint64_t id) {
  if (!v->exact) {
    orc_fixhash_add(v->tab, v->cap, (int32_t)id);
    return;
  }
  kscratch *s = v->s;
  if (s->cnt[id]++ == 0) {
    if (s->ntouched == s->tcap) {
      s->tcap = s->tcap ? 2 * s->tcap : 1024;
      s->touched = (uint64_t *)realloc(s->touched, sizeof(uint64_t) * s->tcap);
    }
    s->touched[s->ntouched++] = id;
  }
}
static void vs_del(vset *v, uint64_t id) {
  if (!v->exact) {
    orc_fixhash_del(v->tab, v->cap, (int32_t)id);
    return;
  }
  if (v->s->cnt[id]) v->s->cnt[id]--;
}
static int vs_test(const vset *v, uint64_t id) {
  return v->exact ? v->s->cnt[id] != 0 : orc_fixhash_test(v->tab, v->cap, (int32_t)id);
}

/* warp_astar_accelerator.h:111-335 for one query (mode REF), or the GB300
 * kernel's specification of it (mode LEX).  Returns the number of vertices in
 * the top-pq list at the end. */
/* Per-hop early-exit features (LEX modes), as the learned search kernel
 * computes them after each hop's select-insert: log2(1 + hops) / 10; the
 * top-k spread (kth - best) and the queue-head gap (head - kth) relative to
 * the progress span |d0 - best| as signed log1p; log2(1 + hops since the
 * top-k set last changed) / 10; log2(1 + distance evaluations) / 10; then the
 * number of changes of the top-k set so far. */
typedef struct {
  int k, trace_hops;
  float *trace; /* trace_hops x ORC_TRACE_FIELDS */
  int32_t version, traced;
} ktrace;

static void trace_hop(ktrace *tr, const kscratch *s, int qn, int ts, float d0, int hops, int evals,
                      int last_change) {
  if (!tr || hops > tr->trace_hops) return;
  const float kth = ts >= tr->k ? s->lt[tr->k - 1].d : s->lt[ts - 1].d;
  const float best = s->lt[0].d;
  const float head = qn > 0 ? s->lq[0].d : kth;
  const float span = fabsf(d0 - best) + 1e-6f * (fabsf(d0) + fabsf(best)) + 1e-30f;
  const float r1 = (kth - best) / span;
  const float r3 = (head - kth) / span;
  float *f = tr->trace + (size_t)(hops - 1) * ORC_TRACE_FIELDS;
  f[0] = log2f(1.0f + (float)hops) * 0.1f;
  f[1] = copysignf(log1pf(fabsf(r1)), r1);
  f[2] = log2f(1.0f + (float)(hops - last_change)) * 0.1f;
  f[3] = copysignf(log1pf(fabsf(r3)), r3);
  f[4] = log2f(1.0f + (float)evals) * 0.1f;
  f[5] = (float)tr->version;
}

/* probes: vertices popped per iteration (warp_astar_accelerator.h:29,
 * 184-232, N_MULTIPROBE; the reference's default is 1).  Only an iteration's
 * first pop takes the finish test; the neighbours of all its pops are
 * filtered before any distance is computed, then select-inserted in order.
 * finish_cnt: the search ends when the finish test has held that many times
 * (FINISH_CNT, :30,190-197,227; default 1); a pop that passes the test
 * before then is processed like any other.  dcheck: the select-insert skips
 * a candidate already in the visited set (__ENABLE_MULTIPROBE_DOUBLE_CHECK,
 * :307-310; off by default), which keeps a vertex listed by two pops of one
 * iteration from entering the queue twice. */
static int ksearch_one(const orc_index *ix, const float *qv, const uint64_t *starts, int ns, int pq, int probes,
                       int finish_cnt, int dcheck, int mode, int use_fma, kscratch *s, uint64_t *out, int32_t *hops_out,
                       int32_t *evals_out, evlog *L, ktrace *tr) {
  const int cap = 8 * pq; /* FixHash<int, TOPK*4*2>, warp_astar_accelerator.h:59-61 */
  const int shift = ix->shift;
  int32_t *tab = s->tab;
  vset vs = {mode == ORC_MODE_LEX_EXACT, tab, cap, s};
  if (vs.exact) {
    for (size_t i = 0; i < s->ntouched; ++i) s->cnt[s->touched[i]] = 0;
    s->ntouched = 0;
  } else {
    orc_fixhash_init(tab, cap);
  }

  int hs = 1, ts = 0; /* REF: SMMH size (+1 dummy slot) and heap size */
  int qn = 0;         /* LEX: queue length (ts shared) */
  int hops = 0, evals = 0;
  int last_change = 0;
  int fin = 0; /* finished[cid] */

  /* :173 the search starts at vertex 0.  Entry points generalise it: the ns
   * start vertices enter the queue (and the visited set) in order before the
   * first pop; d0, the progress reference of the early-exit features, is the
   * first start's distance. */
  float d0 = 0.0f;
  for (int si = 0; si < ns; ++si) {
    const uint64_t start = starts[si];
    const float d = orc_kernel_distance(ix->metric, ix->dim, qv, row(ix, start), use_fma);
    if (si == 0) d0 = d;
    if (mode == ORC_MODE_REF) {
      kp_t e = {(double)d, start};
      smmh_insert(s->q, &hs, e);
    } else {
      lk_t e = {d, 0, start};
      lk_insert(s->lq, &qn, e);
    }
    vs_add(&vs, start);
  }
  evals = ns;

  for (;;) {
    const int avail = mode == ORC_MODE_REF ? hs - 1 : qn; /* :181 while (heap_size > 1) */
    if (avail <= 0) break;
    int m = 0, finished = 0;
    for (int k = 0; k < probes && k < avail; ++k) {
    uint64_t now_id;
    float now_d;
    if (mode == ORC_MODE_REF) {
      kp_t now = smmh_pop_min(s->q, &hs);
      now_id = now.id;
      now_d = (float)now.d;
    } else {
      lk_t now = s->lq[0];
      memmove(s->lq, s->lq + 1, sizeof(lk_t) * (size_t)(qn - 1));
      --qn;
      now_id = now.id;
      now_d = now.d;
    }
    ev(L, ORC_EV_POP, now_id, now_d);
    vs_del(&vs, now_id);
    /* :191 finish test uses <=, on an iteration's first pop only (:190) */
    float tmax = mode == ORC_MODE_REF ? (ts > 0 ? (float)s->t[0].d : 0.0f)
                                      : (ts > 0 ? s->lt[ts - 1].d : 0.0f);
    if (k == 0 && ts == pq && tmax <= now_d && ++fin >= finish_cnt) {
      ev(L, ORC_EV_FINISH, now_id, now_d);
      finished = 1;
      break;
    }
    ++hops;
    /* :198-210 */
    if (mode == ORC_MODE_REF) {
      kp_t e = {(double)now_d, now_id};
      s->t[ts++] = e;
      bh_push(s->t, ts);
      vs_add(&vs, now_id);
      if (ts > pq) {
        kp_t top = s->t[0];
        vs_del(&vs, top.id);
        bh_pop(s->t, ts);
        --ts;
        ev(L, ORC_EV_TEVICT, top.id, (float)top.d);
      }
    } else {
      lk_t e = {now_d, 0, now_id};
      if (tr && (ts < tr->k || lk_less(e, s->lt[tr->k - 1]))) { /* enters the top-k */
        ++tr->version;
        last_change = hops;
      }
      lk_insert(s->lt, &ts, e);
      vs_add(&vs, now_id);
      if (ts > pq) {
        lk_t top = s->lt[ts - 1];
        vs_del(&vs, top.id);
        --ts;
        ev(L, ORC_EV_TEVICT, top.id, top.d);
      }
    }
    /* :211-224 neighbour filter, row order, appended to the iteration's list */
    const uint64_t *grow = ix->graph + (now_id << shift);
    int degree = (int)grow[0];
    for (int i = 1; i <= degree; ++i) {
      uint64_t nb = grow[i];
      if (vs_test(&vs, nb)) continue;
      s->cand[m++] = nb;
    }
    }
    if (finished) break;
    /* :237-287 distances */
    for (int i = 0; i < m; ++i) {
      s->cdist[i] = orc_kernel_distance(ix->metric, ix->dim, qv, row(ix, s->cand[i]), use_fma);
      ev(L, ORC_EV_TEST, s->cand[i], s->cdist[i]);
    }
    evals += m;
    /* :297-322 select-insert, candidate order */
    for (int i = 0; i < m; ++i) {
      float d = s->cdist[i];
      uint64_t id = s->cand[i];
      if (mode == ORC_MODE_REF) {
        if (hs >= pq + 1 && (float)s->q[2].d < d) {
          ev(L, ORC_EV_SKIP, id, d);
          continue;
        }
        if (dcheck && vs_test(&vs, id)) {
          ev(L, ORC_EV_SKIP, id, d);
          continue;
        }
        kp_t e = {(double)d, id};
        smmh_insert(s->q, &hs, e);
        vs_add(&vs, id);
        ev(L, ORC_EV_INSERT, id, d);
        if (hs >= pq + 2) {
          kp_t mx = s->q[2];
          vs_del(&vs, mx.id);
          smmh_pop_max(s->q, &hs);
          ev(L, ORC_EV_QEVICT, mx.id, (float)mx.d);
        }
      } else {
        if (qn >= pq && s->lq[qn - 1].d < d) {
          ev(L, ORC_EV_SKIP, id, d);
          continue;
        }
        if (dcheck && vs_test(&vs, id)) {
          ev(L, ORC_EV_SKIP, id, d);
          continue;
        }
        lk_t e = {d, 0, id};
        lk_insert(s->lq, &qn, e);
        vs_add(&vs, id);
        ev(L, ORC_EV_INSERT, id, d);
        if (qn >= pq + 1) {
          lk_t mx = s->lq[qn - 1];
          vs_del(&vs, mx.id);
          --qn;
          ev(L, ORC_EV_QEVICT, mx.id, mx.d);
        }
      }
    }
    if (mode != ORC_MODE_REF) trace_hop(tr, s, qn, ts, d0, hops, evals, last_change);
  }
  if (tr) tr->traced = hops < tr->trace_hops ? hops : tr->trace_hops;

  /* :331-335 output, ascending.  With fewer than pq popped vertices the
   * reference reads before its heap array (undefined); both modes put the
   * popped vertices first and ORC_NO_ID after. */
  for (int i = 0; i < pq; ++i) out[i] = ORC_NO_ID;
  if (mode == ORC_MODE_REF) {
    int filled = ts;
    for (int i = 0; i < filled; ++i) {
      kp_t e = bh_pop(s->t, filled - i);
      s->tmp_out[filled - 1 - i] = e.id;
      s->cdist[0] = (float)e.d; /* scratch, unused */
    }
    /* Re-derive distances for the log from the output order. */
    for (int i = 0; i < filled; ++i) {
      out[i] = s->tmp_out[i];
      if (L) ev(L, ORC_EV_OUT, out[i], orc_kernel_distance(ix->metric, ix->dim, qv, row(ix, out[i]), use_fma));
    }
  } else {
    for (int i = 0; i < ts; ++i) {
      out[i] = s->lt[i].id;
      ev(L, ORC_EV_OUT, s->lt[i].id, s->lt[i].d);
    }
  }
  if (hops_out) *hops_out = hops;
  if (evals_out) *evals_out = evals;
  return ts;
}

/* ------------------------------------------------------------------------- */
/* Thread pool helper                                                         */
/* ------------------------------------------------------------------------- */

typedef struct {
  const orc_index *ix;
  const float *queries;
  int nq, pq, mode, use_fma;
  uint64_t *out;
  int32_t *hops, *evals, *popped;
  volatile int next;
  volatile int err;
  int k;
  int32_t *explored;
  const uint64_t *starts;
  int ns;
  int probes, finish_cnt, dcheck;
} job_t;

static int maxdeg_of(const orc_index *ix) { return (1 << ix->shift) - 1; }

static void *kworker(void *arg) {
  job_t *j = (job_t *)arg;
  kscratch s;
  if (kscratch_init(&s, j->pq, maxdeg_of(j->ix), j->ix->n) != 0) {
    j->err = 1;
    kscratch_free(&s);
    return NULL;
  }
  for (;;) {
    int i = __sync_fetch_and_add(&j->next, 1);
    if (i >= j->nq) break;
    int32_t h = 0, e = 0;
    const uint64_t zero = 0;
    int ts = ksearch_one(j->ix, j->queries + (size_t)i * (size_t)j->ix->dim,
                         j->starts ? j->starts + (size_t)i * (size_t)j->ns : &zero, j->starts ? j->ns : 1,
                         j->pq, j->probes, j->finish_cnt, j->dcheck, j->mode, j->use_fma, &s, j->out + (size_t)i * (size_t)j->pq, &h, &e,
                         NULL, NULL);
    if (j->hops) j->hops[i] = h;
    if (j->evals) j->evals[i] = e;
    if (j->popped) j->popped[i] = ts;
  }
  kscratch_free(&s);
  return NULL;
}

static int check_index(const orc_index *ix) {
  if (!ix || !ix->data || !ix->graph || ix->n == 0 || ix->dim <= 0) return -1;
  if (ix->shift < 1 || ix->shift > 12) return -1;
  if (ix->metric < ORC_L2 || ix->metric > ORC_HAMMING) return -1;
  return 0;
}

static int run_pool(void *(*fn)(void *), job_t *j, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  int started = 0;
  for (int t = 0; t < nthreads; ++t) {
    if (pthread_create(&th[t], NULL, fn, j) != 0) break;
    ++started;
  }
  if (started == 0) fn(j);
  for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
  return j->err ? -1 : 0;
}

int orc_kernel_search(const orc_index *ix, const float *queries, int nq, int pq, int mode,
                      int use_fma, uint64_t *out, int32_t *hops, int32_t *evals,
                      int32_t *popped, int nthreads) {
  return orc_kernel_search_from(ix, queries, nq, NULL, 1, pq, mode, use_fma, out, hops, evals, popped, nthreads);
}

int orc_kernel_search_from(const orc_index *ix, const float *queries, int nq, const uint64_t *starts, int ns,
                           int pq, int mode, int use_fma, uint64_t *out, int32_t *hops, int32_t *evals,
                           int32_t *popped, int nthreads) {
  return orc_kernel_search_multi(ix, queries, nq, starts, ns, pq, 1, 1, 0, mode, use_fma, out, hops, evals,
                                 popped, nthreads);
}

int orc_kernel_search_multi(const orc_index *ix, const float *queries, int nq, const uint64_t *starts, int ns,
                            int pq, int probes, int finish_cnt, int double_check, int mode, int use_fma,
                            uint64_t *out,
                            int32_t *hops, int32_t *evals, int32_t *popped, int nthreads) {
  if (check_index(ix) || !queries || !out || nq < 0 || pq < 2 || pq > 4095) return -1;
  if (probes < 1 || probes > ORC_MAX_PROBES || finish_cnt < 1) return -1;
  if (mode != ORC_MODE_REF && mode != ORC_MODE_LEX && mode != ORC_MODE_LEX_EXACT) return -1;
  job_t j;
  memset(&j, 0, sizeof j);
  j.ix = ix;
  j.queries = queries;
  j.nq = nq;
  j.pq = pq;
  j.mode = mode;
  j.use_fma = use_fma;
  j.out = out;
  j.hops = hops;
  j.evals = evals;
  j.popped = popped;
  j.starts = starts;
  j.ns = ns;
  j.probes = probes;
  j.finish_cnt = finish_cnt;
  j.dcheck = double_check != 0;
  if (starts) {
    if (ns < 1 || ns > pq) return -1;
    for (size_t i = 0; i < (size_t)nq * (size_t)ns; ++i)
      if (starts[i] >= ix->n) return -1;
  }
  return run_pool(kworker, &j, nthreads);
}

int orc_kernel_search_log(const orc_index *ix, const float *query, int pq, int mode, int use_fma,
                          uint64_t *out, orc_event *log, int cap, int *n_events) {
  return orc_kernel_search_log_multi(ix, query, pq, 1, 1, 0, mode, use_fma, out, log, cap, n_events);
}

int orc_kernel_search_log_multi(const orc_index *ix, const float *query, int pq, int probes, int finish_cnt,
                                int double_check, int mode, int use_fma, uint64_t *out, orc_event *log, int cap, int *n_events) {
  if (check_index(ix) || !query || !out || pq < 2 || pq > 4095) return -1;
  if (probes < 1 || probes > ORC_MAX_PROBES || finish_cnt < 1) return -1;
  kscratch s;
  if (kscratch_init(&s, pq, maxdeg_of(ix), ix->n) != 0) {
    kscratch_free(&s);
    return -1;
  }
  evlog L = {log, cap, 0};
  const uint64_t zero = 0;
  ksearch_one(ix, query, &zero, 1, pq, probes, finish_cnt, double_check != 0, mode, use_fma, &s, out, NULL, NULL,
              &L, NULL);
  if (n_events) *n_events = L.n;
  kscratch_free(&s);
  return 0;
}

int orc_kernel_search_trace(const orc_index *ix, const float *query, int pq, int k, int mode,
                            int use_fma, int trace_hops, float *trace, int32_t *final_version,
                            int32_t *traced, uint64_t *out, int32_t *hops, int32_t *evals) {
  if (check_index(ix) || !query || !out || !trace || pq < 2 || pq > 4095 || k < 1 || k > pq ||
      trace_hops < 1 || mode == ORC_MODE_REF)
    return -1;
  kscratch s;
  if (kscratch_init(&s, pq, maxdeg_of(ix), ix->n) != 0) {
    kscratch_free(&s);
    return -1;
  }
  ktrace tr = {k, trace_hops, trace, 0, 0};
  const uint64_t zero = 0;
  ksearch_one(ix, query, &zero, 1, pq, 1, 1, 0, mode, use_fma, &s, out, hops, evals, NULL, &tr);
  if (final_version) *final_version = tr.version;
  if (traced) *traced = tr.traced;
  kscratch_free(&s);
  return 0;
}

int orc_classify(const orc_event *a, int na, const orc_event *b, int nb, int *at) {
  int n = na < nb ? na : nb;
  for (int i = 0; i < n; ++i) {
    int same = a[i].kind == b[i].kind && a[i].id == b[i].id && a[i].dist == b[i].dist;
    if (same) continue;
    if (at) *at = i;
    if (a[i].kind == b[i].kind && a[i].dist == b[i].dist && a[i].id != b[i].id) return 1;
    return 2;
  }
  if (na != nb) {
    if (at) *at = n;
    return 2;
  }
  if (at) *at = -1;
  return 0;
}

/* ------------------------------------------------------------------------- */
/* CPU best-first search, graph.h:169-216                                     */
/* ------------------------------------------------------------------------- */

typedef struct {
  double d;
  uint64_t id;
} pr_t;

/* std::pair ordering: distance, then id. */
static inline int pr_less(pr_t a, pr_t b) { return a.d < b.d || (a.d == b.d && a.id < b.id); }

/* Binary heaps; 'minh' keeps the smallest pair on top, 'maxh' the largest. */
static void heap_push(pr_t *h, int *n, pr_t e, int ismax) {
  int i = (*n)++;
  h[i] = e;
  while (i > 0) {
    int p = (i - 1) >> 1;
    int up = ismax ? pr_less(h[p], h[i]) : pr_less(h[i], h[p]);
    if (!up) break;
    pr_t t = h[p];
    h[p] = h[i];
    h[i] = t;
    i = p;
  }
}

static pr_t heap_pop(pr_t *h, int *n, int ismax) {
  pr_t top = h[0];
  h[0] = h[--(*n)];
  int i = 0;
  for (;;) {
    int l = 2 * i + 1, r = l + 1, best = i;
    if (l < *n && (ismax ? pr_less(h[best], h[l]) : pr_less(h[l], h[best]))) best = l;
    if (r < *n && (ismax ? pr_less(h[best], h[r]) : pr_less(h[r], h[best]))) best = r;
    if (best == i) break;
    pr_t t = h[best];
    h[best] = h[i];
    h[i] = t;
    i = best;
  }
  return top;
}

typedef struct {
  pr_t *q;
  int qcap;
  pr_t *t;
  uint8_t *visited; /* one byte per vertex, cleared through 'touched' */
  uint64_t *touched;
  size_t ntouched, tcap;
} cscratch;

static int grow_q(cscratch *s, int need) {
  if (need <= s->qcap) return 0;
  int nc = s->qcap ? s->qcap : 1024;
  while (nc < need) nc *= 2;
  pr_t *nq = (pr_t *)realloc(s->q, sizeof(pr_t) * (size_t)nc);
  if (!nq) return -1;
  s->q = nq;
  s->qcap = nc;
  return 0;
}

static int touch(cscratch *s, uint64_t id) {
  if (s->ntouched == s->tcap) {
    size_t nc = s->tcap ? s->tcap * 2 : 4096;
    uint64_t *nt = (uint64_t *)realloc(s->touched, sizeof(uint64_t) * nc);
    if (!nt) return -1;
    s->touched = nt;
    s->tcap = nc;
  }
  s->touched[s->ntouched++] = id;
  s->visited[id] = 1;
  return 0;
}

static int csearch_one(const orc_index *ix, const float *qv, int k, cscratch *s, uint64_t *out,
                       int32_t *explored) {
  int qn = 0, tn = 0;
  const int shift = ix->shift;
  s->ntouched = 0;
  if (ix->n > 0) {
    if (touch(s, 0)) return -1;
    if (grow_q(s, 1)) return -1;
    pr_t e = {orc_cpu_distance(ix->metric, ix->dim, row(ix, 0), qv), 0};
    heap_push(s->q, &qn, e, 0);
  }
  int explore = 0;
  for (int iter = 0; iter < 1000000 && qn > 0; ++iter) {
    pr_t now = s->q[0];
    if (tn == k && s->t[0].d < now.d) break; /* graph.h:188 uses < */
    ++explore;
    heap_pop(s->q, &qn, 0);
    heap_push(s->t, &tn, now, 1);
    if (tn > k) heap_pop(s->t, &tn, 1);
    const uint64_t *grow = ix->graph + (now.id << shift);
    uint64_t degree = grow[0];
    for (uint64_t i = 0; i < degree; ++i) {
      uint64_t nb = grow[i + 1];
      if (s->visited[nb]) continue;
      if (grow_q(s, qn + 1)) return -1;
      pr_t e = {orc_cpu_distance(ix->metric, ix->dim, row(ix, nb), qv), nb};
      heap_push(s->q, &qn, e, 0);
      if (touch(s, nb)) return -1;
    }
  }
  for (int i = 0; i < k; ++i) out[i] = ORC_NO_ID;
  int len = tn;
  for (int i = len - 1; i >= 0; --i) out[i] = heap_pop(s->t, &tn, 1).id;
  for (size_t i = 0; i < s->ntouched; ++i) s->visited[s->touched[i]] = 0;
  if (explored) *explored = explore;
  return 0;
}

static void *cworker(void *arg) {
  job_t *j = (job_t *)arg;
  cscratch s;
  memset(&s, 0, sizeof s);
  s.t = (pr_t *)malloc(sizeof(pr_t) * (size_t)(j->k + 2));
  s.visited = (uint8_t *)calloc((size_t)j->ix->n, 1);
  if (!s.t || !s.visited) {
    j->err = 1;
  } else {
    for (;;) {
      int i = __sync_fetch_and_add(&j->next, 1);
      if (i >= j->nq) break;
      int32_t ex = 0;
      if (csearch_one(j->ix, j->queries + (size_t)i * (size_t)j->ix->dim, j->k, &s,
                      j->out + (size_t)i * (size_t)j->k, &ex)) {
        j->err = 1;
        break;
      }
      if (j->explored) j->explored[i] = ex;
    }
  }
  free(s.q);
  free(s.t);
  free(s.visited);
  free(s.touched);
  return NULL;
}

int orc_cpu_search(const orc_index *ix, const float *queries, int nq, int k, uint64_t *out,
                   int32_t *explored, int nthreads) {
  if (check_index(ix) || !queries || !out || nq < 0 || k < 1) return -1;
  job_t j;
  memset(&j, 0, sizeof j);
  j.ix = ix;
  j.queries = queries;
  j.nq = nq;
  j.k = k;
  j.out = out;
  j.explored = explored;
  return run_pool(cworker, &j, nthreads);
}

int orc_nearest_entry(const orc_index *ix, const float *queries, int nq, const uint64_t *entries, int ne,
                      int ns, int use_fma, uint64_t *starts) {
  if (check_index(ix) || !queries || !entries || !starts || ne < 1 || ns < 1 || ns > ne) return -1;
  for (int e = 0; e < ne; ++e)
    if (entries[e] >= ix->n) return -1;
  float *bd = (float *)malloc(sizeof(float) * (size_t)ns);
  if (!bd) return -1;
  for (int i = 0; i < nq; ++i) {
    const float *q = queries + (size_t)i * (size_t)ix->dim;
    uint64_t *bi = starts + (size_t)i * (size_t)ns;
    int have = 0; /* ascending (distance, id) list of the best `have` */
    for (int e = 0; e < ne; ++e) {
      const float d = orc_kernel_distance(ix->metric, ix->dim, q, row(ix, entries[e]), use_fma);
      const uint64_t id = entries[e];
      int pos = have;
      while (pos > 0 && (d < bd[pos - 1] || (d == bd[pos - 1] && id < bi[pos - 1]))) --pos;
      if (pos >= ns) continue;
      int last = have < ns ? have : ns - 1;
      for (int m = last; m > pos; --m) {
        bd[m] = bd[m - 1];
        bi[m] = bi[m - 1];
      }
      bd[pos] = d;
      bi[pos] = id;
      if (have < ns) ++have;
    }
  }
  free(bd);
  return 0;
}

/* Two-level entry choice.  Entries ids[0..coarse-1] are the coarse entries;
 * each forms its own cluster, and every other entry joins the cluster of its
 * nearest coarse entry (kernel distance, the entry's FP32 row as the query,
 * ties to the smaller id).  A query probes its `probes` nearest coarse
 * entries and starts from the `ns` nearest entries of those clusters
 * (ascending by (distance, id); ns <= probes).  Both steps run on nthreads
 * threads; every result is a per-query (or per-entry) minimum under a total
 * order, so the thread count does not change it. */
typedef struct {
  const orc_index *ix;
  const float *queries;
  int nq;
  const uint64_t *entries;
  int ne, coarse, probes, ns, use_fma;
  int *cl;            /* ne: coarse position of each entry's cluster */
  const int *cstart;  /* coarse + 1: cluster c's entries are members[cstart[c] .. cstart[c+1]) */
  const uint64_t *members;
  uint64_t *starts;
  volatile int next;
  volatile int err;
} twolevel_job;

static void *tl_assign_worker(void *arg) {
  twolevel_job *j = (twolevel_job *)arg;
  for (;;) {
    const int f = __sync_fetch_and_add(&j->next, 1);
    if (f >= j->ne) break;
    if (f < j->coarse) {
      j->cl[f] = f;
      continue;
    }
    uint64_t best;
    if (orc_nearest_entry(j->ix, row(j->ix, j->entries[f]), 1, j->entries, j->coarse, 1, j->use_fma, &best) != 0) {
      j->err = 1;
      break;
    }
    int c = 0;
    while (j->entries[c] != best) ++c; /* the coarse position of that id */
    j->cl[f] = c;
  }
  return NULL;
}

static void *tl_query_worker(void *arg) {
  twolevel_job *j = (twolevel_job *)arg;
  uint64_t *pc = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)j->probes);
  uint64_t *cand = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)j->ne);
  if (!pc || !cand) {
    j->err = 1;
    free(pc);
    free(cand);
    return NULL;
  }
  for (;;) {
    const int i = __sync_fetch_and_add(&j->next, 1);
    if (i >= j->nq) break;
    const float *q = j->queries + (size_t)i * (size_t)j->ix->dim;
    if (orc_nearest_entry(j->ix, q, 1, j->entries, j->coarse, j->probes, j->use_fma, pc) != 0) {
      j->err = 1;
      break;
    }
    int nc = 0;
    for (int p = 0; p < j->probes; ++p) {
      int c = 0;
      while (j->entries[c] != pc[p]) ++c;
      for (int m = j->cstart[c]; m < j->cstart[c + 1]; ++m) cand[nc++] = j->members[m];
    }
    if (orc_nearest_entry(j->ix, q, 1, cand, nc, j->ns, j->use_fma, j->starts + (size_t)i * (size_t)j->ns) != 0) {
      j->err = 1;
      break;
    }
  }
  free(pc);
  free(cand);
  return NULL;
}

static int tl_pool(void *(*fn)(void *), twolevel_job *j, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  pthread_t th[256];
  int started = 0;
  j->next = 0;
  for (int t = 0; t < nthreads; ++t) {
    if (pthread_create(&th[t], NULL, fn, j) != 0) break;
    ++started;
  }
  if (started == 0) fn(j);
  for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
  return j->err ? -1 : 0;
}

int orc_nearest_entry_2level(const orc_index *ix, const float *queries, int nq, const uint64_t *entries, int ne,
                             int coarse, int probes, int ns, int use_fma, uint64_t *starts, int nthreads) {
  if (check_index(ix) || !queries || !entries || !starts || ne < 1 || coarse < 1 || coarse > ne || probes < 1 ||
      probes > coarse || ns < 1 || ns > probes)
    return -1;
  for (int e = 0; e < ne; ++e)
    if (entries[e] >= ix->n) return -1;
  int *cl = (int *)malloc(sizeof(int) * (size_t)ne);
  int *cstart = (int *)calloc((size_t)coarse + 1, sizeof(int));
  int *fill = (int *)calloc((size_t)coarse, sizeof(int));
  uint64_t *members = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)ne);
  twolevel_job j;
  memset(&j, 0, sizeof j);
  int rc = -1;
  if (!cl || !cstart || !fill || !members) goto done;
  j.ix = ix;
  j.queries = queries;
  j.nq = nq;
  j.entries = entries;
  j.ne = ne;
  j.coarse = coarse;
  j.probes = probes;
  j.ns = ns;
  j.use_fma = use_fma;
  j.cl = cl;
  j.starts = starts;
  if (tl_pool(tl_assign_worker, &j, nthreads) != 0) goto done;
  /* clusters as contiguous member lists (member order does not matter: the
   * choice is a minimum under (distance, id)) */
  for (int f = 0; f < ne; ++f) cstart[cl[f] + 1]++;
  for (int c = 0; c < coarse; ++c) cstart[c + 1] += cstart[c];
  for (int f = 0; f < ne; ++f) members[cstart[cl[f]] + fill[cl[f]]++] = entries[f];
  j.cstart = cstart;
  j.members = members;
  rc = tl_pool(tl_query_worker, &j, nthreads);
done:
  free(cl);
  free(cstart);
  free(fill);
  free(members);
  return rc;
}

/* ------------------------------------------------------------------------- */
/* Graph builder: FixedDegreeGraph::add_vertex (graph.h:149-167)              */
/* ------------------------------------------------------------------------- */

typedef struct {
  const float *data;
  uint64_t n;
  int dim, metric, shift, search_degree, fixed_degree;
  uint64_t *edges;   /* n << shift: slot 0 = degree, then ids */
  double *edge_dist; /* the distance of each edge, parallel to edges */
} gbuild;

static const float *gb_row(const gbuild *b, uint64_t i) { return b->data + i * (uint64_t)b->dim; }

/* graph.h:98-114: Hoare partition around the middle element. */
static void gb_qsort(gbuild *b, size_t l, size_t r) {
  size_t mid = (l + r) >> 1;
  long long i = (long long)l, j = (long long)r;
  double k = b->edge_dist[mid];
  do {
    while (b->edge_dist[i] < k) ++i;
    while (k < b->edge_dist[j]) --j;
    if (i <= j) {
      double td = b->edge_dist[i];
      b->edge_dist[i] = b->edge_dist[j];
      b->edge_dist[j] = td;
      uint64_t te = b->edges[i];
      b->edges[i] = b->edges[j];
      b->edges[j] = te;
      ++i;
      --j;
    }
  } while (i <= j);
  if ((size_t)i < r) gb_qsort(b, (size_t)i, r);
  if (j >= 0 && l < (size_t)j) gb_qsort(b, l, (size_t)j);
}

/* graph.h:116-124: distances of a row's edges from its vertex, then sorted. */
static void gb_rank_edges(gbuild *b, size_t off) {
  const uint64_t deg = b->edges[off];
  const float *a = gb_row(b, off >> b->shift);
  for (uint64_t i = 0; i < deg; ++i)
    b->edge_dist[off + i + 1] = orc_cpu_distance(b->metric, b->dim, a, gb_row(b, b->edges[off + i + 1]));
  if (deg > 0) gb_qsort(b, off + 1, off + deg);
}

/* graph.h:32-55: a closer vertex replaces the farthest edge of a full row,
 * then bubbles towards the front. */
static void gb_rank_and_switch(gbuild *b, uint64_t v, uint64_t u) {
  const double curr = orc_cpu_distance(b->metric, b->dim, gb_row(b, v), gb_row(b, u));
  const size_t off = (size_t)v << b->shift;
  const size_t last = off + b->edges[off];
  if (curr >= b->edge_dist[last]) return;
  b->edges[last] = u;
  b->edge_dist[last] = curr;
  for (size_t i = last - 1; i > off; --i) {
    if (b->edge_dist[i] > b->edge_dist[i + 1]) {
      double td = b->edge_dist[i];
      b->edge_dist[i] = b->edge_dist[i + 1];
      b->edge_dist[i + 1] = td;
      uint64_t te = b->edges[i];
      b->edges[i] = b->edges[i + 1];
      b->edges[i + 1] = te;
    } else {
      break;
    }
  }
}

/* graph.h:126-137: append while the row has room (ranking it when it fills),
 * afterwards replace the farthest edge if closer. */
static void gb_add_edge(gbuild *b, uint64_t v, uint64_t u) {
  const size_t off = (size_t)v << b->shift;
  if (b->edges[off] < (uint64_t)b->fixed_degree) {
    ++b->edges[off];
    b->edges[off + b->edges[off]] = u;
    if (b->edges[off] == (uint64_t)b->fixed_degree) gb_rank_edges(b, off);
  } else {
    gb_rank_and_switch(b, v, u);
  }
}

/* graph.h:149-167 after the search: the search_degree nearest results become
 * the vertex's edges (ranked), and each of them gets the reverse edge. */
static void gb_apply(gbuild *b, uint64_t v, const uint64_t *nb, int cnt) {
  const int num = cnt < b->search_degree ? cnt : b->search_degree;
  const size_t off = (size_t)v << b->shift;
  b->edges[off] = (uint64_t)num;
  for (int i = 0; i < num; ++i) b->edges[off + i + 1] = nb[i];
  gb_rank_edges(b, off);
  for (int i = 0; i < num; ++i) gb_add_edge(b, nb[i], v);
}

typedef struct {
  const gbuild *b;
  orc_index ix;      /* the graph as it stands before the batch */
  uint64_t a, e;     /* the batch */
  int budget;
  uint64_t *res;     /* (e - a) x budget result ids, ORC_NO_ID past the end */
  volatile uint64_t next;
  volatile int err;
} gbatch;

static void *gb_worker(void *arg) {
  gbatch *j = (gbatch *)arg;
  cscratch s;
  memset(&s, 0, sizeof s);
  s.t = (pr_t *)malloc(sizeof(pr_t) * (size_t)(j->budget + 2));
  s.visited = (uint8_t *)calloc((size_t)j->b->n, 1);
  if (!s.t || !s.visited) {
    j->err = 1;
  } else {
    for (;;) {
      const uint64_t v = __sync_fetch_and_add(&j->next, 1);
      if (v >= j->e) break;
      if (csearch_one(&j->ix, gb_row(j->b, v), j->budget, &s, j->res + (size_t)(v - j->a) * j->budget, NULL)) {
        j->err = 1;
        break;
      }
    }
  }
  free(s.q);
  free(s.t);
  free(s.visited);
  free(s.touched);
  return NULL;
}

int orc_graph_build(const float *data, uint64_t n, int dim, int metric, int shift, int search_degree,
                    int fixed_degree, int budget, int batch_div, int nthreads, uint64_t *graph_out) {
  if (!data || !graph_out || n == 0 || dim <= 0 || metric < ORC_L2 || metric > ORC_COS) return -1;
  if (shift < 1 || shift > 10 || fixed_degree < 1 || fixed_degree > (1 << shift) - 1) return -1;
  if (search_degree < 1 || search_degree > fixed_degree || budget < search_degree || batch_div < 0) return -1;
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  gbuild b;
  b.data = data;
  b.n = n;
  b.dim = dim;
  b.metric = metric;
  b.shift = shift;
  b.search_degree = search_degree;
  b.fixed_degree = fixed_degree;
  b.edges = graph_out;
  memset(graph_out, 0, sizeof(uint64_t) * ((size_t)n << shift));
  b.edge_dist = (double *)calloc((size_t)n << shift, sizeof(double));
  const uint64_t maxb = batch_div > 0 ? (n / (uint64_t)batch_div + 1) : 1;
  uint64_t *res = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)maxb * (size_t)budget);
  if (!b.edge_dist || !res) {
    free(b.edge_dist);
    free(res);
    return -1;
  }
  int rc = 0;
  uint64_t a = 0;
  while (a < n && rc == 0) {
    /* batch_div 0: one vertex at a time (the reference's loop); otherwise
     * max(1, inserted / batch_div) vertices, searched against the graph as
     * it stood before the batch and applied in id order */
    uint64_t bs = batch_div > 0 ? a / (uint64_t)batch_div : 1;
    if (bs < 1) bs = 1;
    const uint64_t e = a + bs < n ? a + bs : n;
    if (a == 0) {
      /* data.h:139-144: the first vertex finds no other vertex */
      for (uint64_t v = a; v < e; ++v) gb_apply(&b, v, res, 0);
      a = e;
      continue;
    }
    gbatch j;
    memset(&j, 0, sizeof j);
    j.b = &b;
    j.ix.data = data;
    j.ix.graph = graph_out;
    j.ix.n = n;
    j.ix.dim = dim;
    j.ix.shift = shift;
    j.ix.metric = metric;
    j.a = a;
    j.e = e;
    j.budget = budget;
    j.res = res;
    j.next = a;
    const uint64_t nt = e - a < (uint64_t)nthreads ? e - a : (uint64_t)nthreads;
    if (nt <= 1) {
      gb_worker(&j);
    } else {
      pthread_t th[256];
      int started = 0;
      for (uint64_t t = 0; t < nt; ++t) {
        if (pthread_create(&th[t], NULL, gb_worker, &j) != 0) break;
        ++started;
      }
      if (started == 0) gb_worker(&j);
      for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
    }
    if (j.err) {
      rc = -1;
      break;
    }
    for (uint64_t v = a; v < e; ++v) {
      const uint64_t *r = res + (size_t)(v - a) * budget;
      int cnt = 0;
      while (cnt < budget && r[cnt] != ORC_NO_ID) ++cnt;
      gb_apply(&b, v, r, cnt);
    }
    a = e;
  }
  free(b.edge_dist);
  free(res);
  return rc;
}

/* ------------------------------------------------------------------------- */
/* 256-bit sign codes (hash_warp_no_heap_astar_accelerator.h:22-41)          */
/* ------------------------------------------------------------------------- */

/* codes[r*8 + i/32] bit i%32 = (x_r . plane_i >= 0), the dot product summed
 * as the kernel sums distances (orc_kernel_distance, inner product: partial
 * sums of lane-strided fused multiply-adds, xor butterfly). */
int orc_hash_codes(const float *rows, uint64_t n, int dim, const float *planes, int use_fma, uint32_t *codes) {
  if (!rows || !planes || !codes || dim <= 0) return -1;
  for (uint64_t r = 0; r < n; ++r) {
    const float *x = rows + r * (uint64_t)dim;
    for (int w = 0; w < 8; ++w) codes[r * 8 + w] = 0u;
    for (int i = 0; i < 256; ++i) {
      const float t = -orc_kernel_distance(ORC_IP, dim, x, planes + (size_t)i * (size_t)dim, use_fma);
      if (t >= 0.0f) codes[r * 8 + (i >> 5)] |= 1u << (i & 31);
    }
  }
  return 0;
}
