/*
 * Host side of libcintgpu: libcint's C ABI for the two-electron hot path plus the batched plan
 * API (include/cintgpu.h).  Everything numerical runs in the CUDA kernels of rys_kernels.cu; this
 * file only plans work:
 *
 *   shells      atm/bas/env are read exactly as libcint does (include/cint.h.in:26-72).  A shell
 *               with nctr > 1 becomes nctr virtual shells, one per contraction column, whose
 *               blocks land at the offsets libcint's c2s_sph_2e1 uses (src/cart2sph.c:5372-5377).
 *   pairs       per ordered shell pair and primitive pair: a_A + a_B, its inverse, the product
 *               centre, K = c_A c_B exp(-a_A a_B/(a_A+a_B) |AB|^2) and libcint's screening value
 *               cce (CINTset_pairdata, src/optimizer.c:288-342, same formula and operation order).
 *               A pair whose every primitive pair is screened makes the quartet empty, like
 *               libcint's NOVALUE pairs (src/cint2e.c:281-285).
 *   tasks       quartets are put in a canonical order (larger l first inside each pair, larger
 *               pair first) for the int2e kinds, cut into primitive-quartet slices by a cost
 *               model, and sorted longest first within three task groups: regular classes,
 *               classes needing 48 KB of shared memory per warp, and int2e classes evaluated
 *               per primitive.
 *   execution   one launch of the warp-per-task kernel per non-empty group (warps take tasks
 *               from an atomic counter; the warp finishing a quartet's last slice transforms
 *               and stores it), then an output kernel for empty quartets (or, for plans that
 *               keep it separate, for every quartet: sum of slices, cart->sph, strided store).
 *
 * Thread safety: the drop-in entry points keep one CUDA stream, device arena and pinned staging
 * buffer per calling thread, so OpenMP callers may call them concurrently (libcint's contract,
 * README.rst:39).  The device tables are initialised once under a mutex.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <cmath>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <functional>
#include <limits>
#include <unordered_map>
#include <vector>

#include "cintgpu.h"
#include "rys_kernels.h"

namespace {

thread_local std::string tl_error;

void set_error(const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    tl_error = buf;
}

#define CUDA_OK(call)                                                                       \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) {                                                            \
            set_error("%s failed: %s", #call, cudaGetErrorString(e_));                      \
            return CINTGPU_ERR_CUDA;                                                        \
        }                                                                                   \
    } while (0)

/* ------------------------------------------------------------------ cart -> sph rows */
double fact(int n) { double f = 1; for (int i = 2; i <= n; i++) f *= i; return f; }
double binom(int n, int k) { return (k < 0 || k > n) ? 0 : fact(n) / (fact(k) * fact(n - k)); }

int cart_index(int l, int lx, int ly)   /* CINTcart_comp order, src/cint_bas.c:166-181 */
{
    int idx = 0;
    for (int x = l; x > lx; x--) idx += l - x + 1;
    return idx + (l - lx - ly);
}

/* Real solid harmonics r^l Y_lm (unit-sphere normalised, m = -l..l) as Cartesian monomials:
 * closed form of the Racah-normalised S_lm (Schlegel & Frisch, IJQC 54 (1995) 83; the
 * convention of libcint src/cart2sph.c:8-10) times sqrt((2l+1)/4pi).  l = 0, 1 are identities
 * because libcint folds their factors into the common factor (src/g1e.c:565-572). */
void c2s_rows(std::vector<int> &nnz, std::vector<int> &idx, std::vector<double> &val)
{
    const int rows = (CG_MAX_SHELL_L + 1) * (CG_MAX_SHELL_L + 1);
    nnz.assign(rows, 0);
    idx.assign(rows * CG_C2S_MAXNNZ, 0);
    val.assign(rows * CG_C2S_MAXNNZ, 0.0);
    for (int l = 2; l <= CG_MAX_SHELL_L; l++) {
        int nc = (l + 1) * (l + 2) / 2;
        std::vector<double> c((2 * l + 1) * nc, 0.0);
        double unit = sqrt((2 * l + 1) / (4 * M_PI));
        for (int m = -l; m <= l; m++) {
            int am = abs(m);
            double N = sqrt(2.0 * fact(l + am) * fact(l - am) / (m == 0 ? 2.0 : 1.0))
                     / (pow(2.0, am) * fact(l));
            for (int t = 0; t <= (l - am) / 2; t++)
                for (int u = 0; u <= t; u++)
                    for (int v2 = (m < 0 ? 1 : 0); v2 <= am; v2 += 2) {
                        int vm2 = m < 0 ? 1 : 0;
                        int sgn = t + (v2 - vm2) / 2;
                        double C = ((sgn & 1) ? -1.0 : 1.0) * pow(0.25, t) * binom(l, t)
                                 * binom(l - t, am + t) * binom(t, u) * binom(am, v2);
                        int px = 2 * t + am - 2 * u - v2, py = 2 * u + v2, pz = l - 2 * t - am;
                        if (px < 0 || py < 0 || pz < 0) continue;
                        c[(m + l) * nc + cart_index(l, px, py)] += unit * N * C;
                    }
        }
        for (int m = 0; m < 2 * l + 1; m++) {
            int row = l * l + m, k = 0;
            for (int p = 0; p < nc; p++) {
                if (c[m * nc + p] != 0.0) {
                    idx[row * CG_C2S_MAXNNZ + k] = p;
                    val[row * CG_C2S_MAXNNZ + k] = c[m * nc + p];
                    k++;
                }
            }
            nnz[row] = k;
        }
    }
}

/* ------------------------------------------------------------------ device context */
struct Global {
    std::mutex mu;
    bool ready = false;
    int status = 0;
    int device = -1;
    int sm_count = 0;
    double *rys_coef = nullptr;
};
Global g_ctx;

int ensure_init()
{
    std::lock_guard<std::mutex> lk(g_ctx.mu);
    if (g_ctx.ready) return g_ctx.status;
    g_ctx.ready = true;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        set_error("no CUDA device: %s", cudaGetErrorString(e));
        g_ctx.status = CINTGPU_ERR_CUDA;
        return g_ctx.status;
    }
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, dev);
    g_ctx.device = dev;
    g_ctx.sm_count = prop.multiProcessorCount;
    std::vector<int> nnz, idx;
    std::vector<double> val;
    c2s_rows(nnz, idx, val);
    int rc = cg_kernels_init(nnz.data(), idx.data(), val.data(), &g_ctx.rys_coef);
    if (rc) {
        set_error("kernel table initialisation failed: %s", cudaGetErrorString((cudaError_t)rc));
        g_ctx.status = CINTGPU_ERR_CUDA;
    }
    return g_ctx.status;
}

/* ------------------------------------------------------------------ shells and pairs */
struct ShellView {
    int l, nprim, nctr, atom;
    double R[3];
    const double *ex, *cf;
};

/* NaN or Inf in a shell's coordinates, exponents or coefficients: rejected with a message (libcint
 * would carry them into its root finder, which exits on failure, src/rys_roots.c:115-121) */
int check_finite(int sh, const ShellView &s)
{
    for (int c = 0; c < 3; c++)
        if (!std::isfinite(s.R[c])) { set_error("shell %d: non-finite coordinate", sh); return CINTGPU_ERR_ARG; }
    for (int i = 0; i < s.nprim; i++)
        if (!std::isfinite(s.ex[i])) { set_error("shell %d: non-finite exponent", sh); return CINTGPU_ERR_ARG; }
    for (int i = 0; i < s.nprim * s.nctr; i++)
        if (!std::isfinite(s.cf[i])) { set_error("shell %d: non-finite coefficient", sh); return CINTGPU_ERR_ARG; }
    return 0;
}

int read_shell(int sh, const int *atm, int natm, const int *bas, const double *env, ShellView *s)
{
    if (sh < 0) { set_error("negative shell index %d", sh); return CINTGPU_ERR_ARG; }
    const int *b = bas + BAS_SLOTS * sh;
    s->l = b[ANG_OF];
    s->nprim = b[NPRIM_OF];
    s->nctr = b[NCTR_OF];
    if (s->l < 0 || s->l > CG_MAX_SHELL_L) {
        set_error("shell %d: angular momentum %d outside 0..%d", sh, s->l, CG_MAX_SHELL_L);
        return CINTGPU_ERR_UNSUPPORTED;
    }
    if (s->nprim < 1 || s->nprim > 64 || s->nctr < 1 || s->nctr > 64) {
        set_error("shell %d: nprim %d / nctr %d outside 1..64", sh, s->nprim, s->nctr);
        return CINTGPU_ERR_ARG;
    }
    int at = b[ATOM_OF];
    if (at < 0 || at >= natm) { set_error("shell %d: atom %d outside 0..%d", sh, at, natm - 1); return CINTGPU_ERR_ARG; }
    s->atom = at;
    const double *r = env + atm[ATM_SLOTS * at + PTR_COORD];
    s->R[0] = r[0]; s->R[1] = r[1]; s->R[2] = r[2];
    s->ex = env + b[PTR_EXP];
    s->cf = env + b[PTR_COEFF];
    return 0;
}

int ncart_l(int l) { return (l + 1) * (l + 2) / 2; }
int nsph_l(int l) { return 2 * l + 1; }

double common_fac_sp(int l)    /* src/g1e.c:565-572 */
{
    return l == 0 ? 0.282094791773878143 : l == 1 ? 0.488602511902919921 : 1.0;
}

/* shell-pair key packed into 60 bits: shell indices + 1 (21 bits each), contraction columns
 * (6 bits each), the l ceiling entering libcint's log_rr (5 bits), pair kind (1 bit) */
inline uint64_t pair_key(int a, int ca, int b, int cb, int lsum, int kind)
{
    return (uint64_t)(a + 1) | ((uint64_t)(b + 1) << 21) | ((uint64_t)ca << 42) | ((uint64_t)cb << 48)
           | ((uint64_t)lsum << 54) | ((uint64_t)kind << 59);
}
const int PAIR_KEY_MAX_SHELL = (1 << 21) - 2;

/* open-addressing map from packed pair keys (never 0) to pair ids */
struct PairMap {
    std::vector<uint64_t> keys;
    std::vector<int> vals;
    size_t mask = 0, n = 0;
    static uint64_t mix(uint64_t x)
    {
        x ^= x >> 33; x *= 0xff51afd7ed558ccdULL;
        x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL;
        return x ^ (x >> 33);
    }
    int find(uint64_t k) const
    {
        if (!mask) return -1;
        for (size_t i = mix(k) & mask;; i = (i + 1) & mask) {
            if (keys[i] == k) return vals[i];
            if (keys[i] == 0) return -1;
        }
    }
    void insert(uint64_t k, int v)
    {
        if (2 * (n + 1) > mask + 1) {
            std::vector<uint64_t> ok;
            std::vector<int> ov;
            ok.swap(keys);
            ov.swap(vals);
            size_t cap = std::max<size_t>(1024, 2 * (mask + 1));
            keys.assign(cap, 0);
            vals.assign(cap, 0);
            mask = cap - 1;
            n = 0;
            for (size_t i = 0; i < ok.size(); i++)
                if (ok[i]) insert(ok[i], ov[i]);
        }
        size_t i = mix(k) & mask;
        while (keys[i]) i = (i + 1) & mask;
        keys[i] = k;
        vals[i] = v;
        n++;
    }
};

}  // namespace

/* ------------------------------------------------------------------ plan */
/* allocator whose resize leaves new elements uninitialised (for tables filled right after) */
template <class T> struct NoInitAlloc : std::allocator<T> {
    template <class U> struct rebind { using other = NoInitAlloc<U>; };
    NoInitAlloc() = default;
    template <class U> NoInitAlloc(const NoInitAlloc<U> &) {}
    template <class U> void construct(U *p) noexcept { ::new ((void *)p) U; }
    template <class U, class... A> void construct(U *p, A &&...a) { ::new ((void *)p) U(std::forward<A>(a)...); }
};

struct TaskGroup {              /* one kernel launch: tasks [task0, task0 + ntasks) */
    int task0 = 0, ntasks = 0;
    int ws = CG_WS_SMALL;       /* shared-memory doubles per warp */
    int blocks_per_sm = 2;
    int nblocks = 1;            /* CTAs of the launch (4 warps each) */
};

struct CINTGPUPlan {
    int kind = 0;
    int mode = CG_MODE_ERI;
    int ncomp = 1;
    int sph = 1;
    int three = 0;                 /* int3c2e and int2c2e: slot 3 is a unit s partner */
    int two = 0;                   /* int2c2e: slot 1 is a unit s partner as well */
    int jmode = 0;                 /* J (bit 0) / K (bit 1) contraction instead of stored integrals */
    int gradj = 0;                 /* J_GRAD(_EXP): contraction-first adjoint kernel (CG_MODE_GRADJ,
                                      CG_MODE_GRADAJ) */
    int nao_cart = 0;
    int natm = 0;
    int64_t nprim_tot = 0;
    double expcutoff = 60;
    double omega2 = 0;             /* omega^2 of the long-range Coulomb (0: 1/r) */
    int64_t nitems = 0;
    int64_t out_size = 0;          /* doubles per component */
    double flops = 0;
    double flops_ref = 0;          /* the same quartets by libcint's per-primitive algorithm */
    int64_t prim_quartets = 0;
    int max_nf = 1;
    /* host images */
    std::vector<CGPair> pairs;
    std::vector<CGPrimPair> prims;
    std::vector<CGTask> tasks;
    std::vector<CGOutTask> outs;
    std::vector<int, NoInitAlloc<int>> pqlist;   /* surviving primitive quartets, per task slice */
    std::vector<CGGradClass> gclass;   /* adjoint iteration tables per class */
    std::vector<CGGradChunk> gchunk;
    std::vector<CGGradEnt> gent;
    std::vector<CGEriClass> eclass;    /* contraction-first tables per class (ERI mode) */
    std::vector<CGEriGroup> egroup;
    std::vector<int> eperm;
    std::vector<int> hprog;        /* horizontal-transfer programs of the classes */
    std::vector<int> eround;       /* stage-3 rounds: start | count << 16 | box << 24 */
    std::vector<int> empty_outs;   /* output quartets without any task (zero-filled) */
    bool fuse_out = true;          /* the integral kernel stores finished quartets itself */
    int plan_threads = 1;          /* host threads for the planner's screening (plans created by
                                      cintgpu_plan_create*; chunk plans are built in parallel) */
    std::vector<int> wide;         /* class keys forced into the 48 KB group (per-class tuning) */
    int ws_kb = 0;                 /* shared memory per warp of the regular group in KB (0: the
                                      CINTGPU_WS_KB override or the default 24) */
    int prim_l = 4;                /* int2e classes with ll >= prim_l (or lj >= prim_l when the
                                      bra route does not take them) transfer per primitive
                                      (CINTGPU_PER_PRIMITIVE_L overrides, 0 = every class) */
    int bra_l = 2;                 /* classes with lj >= bra_l, li + lj >= bra_lsum and ll < prim_l
                                      transfer the bra per term (CINTGPU_BRA_TERM_L overrides, e.g.
                                      99 = never) */
    int bra_lsum = 5;              /* (dd| stays contraction first: measured within 1e-11 of the
                                      long-double referee on c1, where (fd| reaches 2e-10 */
    bool own_slots = false;        /* some tasks accumulate in per-warp slots (CGTask::own_slot) */
    int hrr_max = 1;               /* doubles of one transfer buffer, largest class */
    int nef_max = 1;               /* (e0|f0) accumulators, largest class */
    std::vector<int> out_item;     /* item index of each CGOutTask */
    TaskGroup groups[3];           /* [0] regular classes, [1] classes needing 48 KB per warp,
                                      [2] int2e classes evaluated per primitive (lj or ll >= 4) */
    int64_t gctr_size = 0;
    /* device */
    char *dbuf = nullptr;
    size_t dbuf_size = 0;
    bool owns_dbuf = true;
    CGPair *d_pairs = nullptr;
    CGPrimPair *d_prims = nullptr;
    CGTask *d_tasks = nullptr;
    CGOutTask *d_outs = nullptr;
    int *d_pqlist = nullptr;
    CGGradClass *d_gclass = nullptr;
    CGGradChunk *d_gchunk = nullptr;
    CGGradEnt *d_gent = nullptr;
    CGEriClass *d_eclass = nullptr;
    CGEriGroup *d_egroup = nullptr;
    int *d_eperm = nullptr;
    int *d_hprog = nullptr;
    int *d_eround = nullptr;
    int *d_empty = nullptr;
    int *d_done = nullptr;         /* finished slices per output quartet (fused output) */
    double *d_oscr = nullptr;      /* per-warp transform scratch of the integral kernel */
    double *d_wslot = nullptr;     /* per-warp slots of own-slot tasks */
    double *cur_out = nullptr;
    double *d_gctr = nullptr;
    int *d_counters = nullptr;     /* [0], [1], [3]: task counters of groups 0, 1, 2; [2]: status */
    int *d_nonempty = nullptr;
    double *d_scratch = nullptr;
    int out_blocks = 1;
    int64_t scratch_per_warp = 0;
    double *d_wscratch = nullptr;  /* per-warp accumulators of the J contraction */
    const double *cur_dm = nullptr;  /* density / J / gradient of the execution being enqueued */
    double *cur_vj = nullptr;
    double *cur_vk = nullptr;
    double *cur_grad = nullptr, *cur_galpha = nullptr;
    int64_t wscratch_stride = 0;
    int wscratch_warps = 0;
    cudaStream_t side = nullptr;   /* second stream for the large-class group */
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaEvent_t ev_t0 = nullptr, ev_t1 = nullptr;   /* around the compute kernels (timing) */
    bool timed = false;            /* ev_t0/ev_t1 recorded at least once */
};

namespace {

/* What an optimizer (int2e_optimizer & co.) keeps for the drop-in calls made with it: the shell
 * pairs' primitive data (libcint's PairData, src/optimizer.c:288-342: product centres, screening
 * values, prefactors), built on first use and shared by every thread calling with the same
 * CINTOpt, which saves each later call that pair work.  Lives in a side table keyed by the
 * CINTOpt pointer and is freed by CINTdel_optimizer. */
struct OptPair {
    CGPair pair;
    std::vector<CGPrimPair> prims;
    bool empty;
};
struct OptState {
    std::mutex mu;
    /* by primitive cutoff (int2e 61, int3c2e 60 by default), then pair_key */
    std::map<double, std::unordered_map<uint64_t, std::unique_ptr<OptPair>>> pairs;
};
std::mutex g_opt_mu;
std::unordered_map<const void *, std::shared_ptr<OptState>> g_opt_states;

std::shared_ptr<OptState> opt_state(const void *opt)
{
    if (!opt) return nullptr;
    std::lock_guard<std::mutex> lk(g_opt_mu);
    auto it = g_opt_states.find(opt);
    return it == g_opt_states.end() ? nullptr : it->second;
}

struct Builder {
    CINTGPUPlan *P;
    const int *atm;
    int natm;
    const int *bas;
    const double *env;
    PairMap pair_index;
    std::vector<char> pair_empty;
    std::vector<std::vector<double>> logmaxc;   /* per original shell index (empty: not yet) */
    const std::vector<int> *ao_loc = nullptr;     /* Cartesian AO offset per shell (J/adjoint) */
    const std::vector<int> *prim_loc = nullptr;   /* first primitive per shell (J/adjoint) */
    OptState *opt = nullptr;                      /* optimizer pair cache (drop-in calls) */

    void locate(CGPair &p, int sa, const ShellView &A, int ca, int sb, const ShellView &B, int cb)
    {
        p.atom_a = A.atom; p.atom_b = B.atom;
        p.ao_a = p.ao_b = p.gp_a = p.gp_b = 0;
        if (ao_loc && sa >= 0 && sa < (int)ao_loc->size()) {
            p.ao_a = (*ao_loc)[sa] + ca * ncart_l(A.l);
            p.gp_a = (*prim_loc)[sa];
        }
        if (ao_loc && sb >= 0 && sb < (int)ao_loc->size()) {
            p.ao_b = (*ao_loc)[sb] + cb * ncart_l(B.l);
            p.gp_b = (*prim_loc)[sb];
        }
    }

    /* the returned data stay valid while the cache grows (inner buffers move with their vectors) */
    const double *log_maxc(int sh, const ShellView &s)
    {
        if ((size_t)sh >= logmaxc.size()) logmaxc.resize((size_t)sh + 1);
        std::vector<double> &v = logmaxc[sh];
        if (!v.empty()) return v.data();
        v.resize(s.nprim);
        for (int ip = 0; ip < s.nprim; ip++) {     /* CINTOpt_log_max_pgto_coeff, :248-259 */
            double m = 0;
            for (int c = 0; c < s.nctr; c++) m = std::max(m, fabs(s.cf[c * s.nprim + ip]));
            v[ip] = log(m);
        }
        return v.data();
    }

    /* ordered pair (A col ca, B col cb); lsum = l ceilings entering libcint's log_rr */
    int pair(int sa, const ShellView &A, int ca, int sb, const ShellView &B, int cb, int lsum)
    {
        const uint64_t key = pair_key(sa, ca, sb, cb, lsum, 0);
        const int found = pair_index.find(key);
        if (found >= 0) return found;
        if (opt) {
            OptPair *e = nullptr;
            {
                std::lock_guard<std::mutex> lk(opt->mu);
                auto &m = opt->pairs[P->expcutoff];
                auto it = m.find(key);
                if (it != m.end()) e = it->second.get();
            }
            if (!e) {   /* build it in a scratch plan and publish it (entries never change) */
                CINTGPUPlan scratch;
                scratch.expcutoff = P->expcutoff;
                Builder b2{&scratch, atm, natm, bas, env, {}, {}, {}};
                const int id = b2.pair(sa, A, ca, sb, B, cb, lsum);
                auto n = std::make_unique<OptPair>();
                n->pair = scratch.pairs[id];
                n->prims.assign(scratch.prims.begin(), scratch.prims.end());
                n->empty = b2.pair_empty[id] != 0;
                std::lock_guard<std::mutex> lk(opt->mu);
                e = opt->pairs[P->expcutoff].emplace(key, std::move(n)).first->second.get();
            }
            CGPair p = e->pair;
            p.prim_off = (int)P->prims.size();
            P->prims.insert(P->prims.end(), e->prims.begin(), e->prims.end());
            const int id = (int)P->pairs.size();
            P->pairs.push_back(p);
            pair_empty.push_back(e->empty ? 1 : 0);
            pair_index.insert(key, id);
            return id;
        }
        CGPair p;
        for (int c = 0; c < 3; c++) { p.AB[c] = A.R[c] - B.R[c]; p.A[c] = A.R[c]; }
        p.prim_off = (int)P->prims.size();
        p.npa = A.nprim; p.npb = B.nprim; p.la = A.l; p.lb = B.l; p.pad = 0;
        locate(p, sa, A, ca, sb, B, cb);
        double rr = p.AB[0] * p.AB[0] + p.AB[1] * p.AB[1] + p.AB[2] * p.AB[2];
        /* CINTset_pairdata, src/optimizer.c:288-342 */
        double aij_last = A.ex[A.nprim - 1] + B.ex[B.nprim - 1];
        double log_rr = 1.7 - 1.5 * log(aij_last);
        if (lsum > 0) log_rr += lsum * log(sqrt(rr) + 1.);
        const double *lca = log_maxc(sa, A);
        const double *lcb = log_maxc(sb, B);
        bool empty = true;
        for (int jp = 0; jp < B.nprim; jp++)
            for (int ip = 0; ip < A.nprim; ip++) {
                CGPrimPair q;
                double ai = A.ex[ip], aj = B.ex[jp];
                double inv = 1 / (ai + aj);
                double eij = rr * ai * aj * inv;
                double cce = eij - log_rr - lca[ip] - lcb[jp];
                q.a = ai + aj;
                q.inv_a = 1.0 / q.a;
                q.cce = cce;
                q.aA = ai;
                if (cce < P->expcutoff) {
                    empty = false;
                    double wj = aj * inv;
                    for (int c = 0; c < 3; c++) q.P[c] = A.R[c] + wj * (B.R[c] - A.R[c]);
                    q.K = A.cf[ca * A.nprim + ip] * B.cf[cb * B.nprim + jp] * exp(-eij);
                } else {
                    /* libcint keeps eij = 0 for such pairs; they contribute exactly zero */
                    for (int c = 0; c < 3; c++) q.P[c] = A.R[c];
                    q.K = 0.0;
                }
                P->prims.push_back(q);
            }
        int id = (int)P->pairs.size();
        P->pairs.push_back(p);
        pair_empty.push_back(empty ? 1 : 0);
        pair_index.insert(key, id);
        return id;
    }

    /* the ket of int3c2e: shell k with a zero-exponent s partner; no ket screening */
    int single(int sk, const ShellView &K, int ck)
    {
        const uint64_t key = pair_key(sk, ck, -1, 0, 0, 1);
        const int found = pair_index.find(key);
        if (found >= 0) return found;
        CGPair p;
        for (int c = 0; c < 3; c++) { p.AB[c] = 0.0; p.A[c] = K.R[c]; }
        p.prim_off = (int)P->prims.size();
        p.npa = K.nprim; p.npb = 1; p.la = K.l; p.lb = 0; p.pad = 0;
        locate(p, sk, K, ck, -1, K, 0);
        for (int kp = 0; kp < K.nprim; kp++) {
            CGPrimPair q;
            q.a = K.ex[kp];
            q.inv_a = 1.0 / q.a;
            for (int c = 0; c < 3; c++) q.P[c] = K.R[c];
            q.K = K.cf[ck * K.nprim + kp];
            q.cce = 0.0;
            q.aA = K.ex[kp];
            P->prims.push_back(q);
        }
        int id = (int)P->pairs.size();
        P->pairs.push_back(p);
        pair_empty.push_back(0);
        pair_index.insert(key, id);
        return id;
    }
};

/* libcint's per-primitive algorithm for one surviving primitive quartet of an int2e class (FMA =
 * 2): per root, coefficient setup 20, VRR 15 per (e, f) entry, 2 per HRR entry written and axis,
 * gout 3 per Cartesian component (src/g2e.c:272-693, src/cint2e.c:961-1183) */
double flops_libcint_primq(int li, int lj, int lk, int ll)
{
    CGLayout L;
    cg_layout(li, lj, lk, ll, CG_MODE_ERI, CG_WS_MAX, &L);
    double hrr = 0;
    for (int j = 1; j < L.dJ; j++) hrr += (L.nmax - j + 1) * (L.mmax + 1);
    for (int l = 1; l < L.dL; l++) hrr += L.dI * L.dJ * (L.mmax - l + 1);
    double vrr = (double)(L.nmax + 1) * (L.mmax + 1);
    return L.nroots * (20 + 3 * 5 * vrr + 3 * 2 * hrr + 3.0 * L.nf);
}

/* algorithmic FP64 flop model per surviving primitive quartet (FMA = 2) */
double flops_per_primq(int li, int lj, int lk, int ll, int mode)
{
    CGLayout L;
    cg_layout(li, lj, lk, ll, mode, CG_WS_MAX, &L);
    int n = L.nroots;
    double hrr = 0;
    for (int j = 1; j < L.dJ; j++) hrr += (L.nmax - j + 1) * (L.mmax + 1);
    for (int l = 1; l < L.dL; l++) hrr += L.dI * L.dJ * (L.mmax - l + 1);
    double vrr = (double)(L.nmax + 1) * (L.mmax + 1);
    if (mode == CG_MODE_ERI) {
        /* contraction first: VRR, then per group one product and 2 flops per member; the
         * transfer is per contracted quartet and not counted */
        auto nc = [](int l) { return (l + 1) * (l + 2) / 2; };
        auto range = [&](int l0, int l1) { int t = 0; for (int l = l0; l <= l0 + l1; l++) t += nc(l); return t; };
        double ngroup = (double)nc(li + lj) * nc(lk + ll);
        double nef = (double)range(li, lj) * range(lk, ll);
        return n * (20 + 3 * 5 * vrr + ngroup + 2 * nef);
    }
    if (mode == CG_MODE_ERIB) {
        /* bra per term: VRR, the bra transfer of each axis, then per (ij, fx, fy) group one
         * product and 2 flops per f member; the ket transfer is per contracted quartet */
        auto nc = [](int l) { return (l + 1) * (l + 2) / 2; };
        double hrr_bra = 0;
        for (int j = 1; j <= lj; j++) hrr_bra += (double)(li + lj - j + 1) * (lk + ll + 1);
        double vrr2 = (double)(li + lj + 1) * (lk + ll + 1);
        double nij = (double)nc(li) * nc(lj);
        double nfr = 0;
        for (int l = lk; l <= lk + ll; l++) nfr += nc(l);
        return n * (20 + 3 * 5 * vrr2 + 3 * 2 * hrr_bra + nij * nc(lk + ll) + 2 * nij * nfr);
    }
    if (mode == CG_MODE_GRADJ || mode == CG_MODE_GRADAJ) {
        /* contraction-first adjoint: VRR to (li+lj+d, lk+ll+d); per side three contractions
         * (z, y, x; 2 flops per product) and the sums over terms (bra: 3 per e', ket: 2 per f';
         * with exponents 4 more per entry and the per-term warp sums; the derivative weights are
         * per task and not counted) */
        auto nc = [](int l) { return (l + 1) * (l + 2) / 2; };
        auto np2 = [](int l) { return (l + 1) * (l + 2) / 2.0; };
        auto ntet = [](int l) { return l < 0 ? 0.0 : (l + 1) * (l + 2) * (l + 3) / 6.0; };
        const int Le = li + lj, Lf = lk + ll, d = mode == CG_MODE_GRADAJ ? 2 : 1;
        double nE = 0, nF = 0;
        for (int l = li; l <= Le; l++) nE += nc(l);
        for (int l = lk; l <= Lf; l++) nF += nc(l);
        const double na = Le + d + 1, nm = Lf + d + 1;
        const double nEp = ntet(Le + d) - ntet(li - 2), nFp = ntet(Lf + d) - ntet(lk - 2);
        const double xs = d == 2 ? 4 : 0;
        const double bra = 2 * nF * na + 2 * np2(Le + d) * np2(Lf) + nEp * (2 * (Lf + 1) + 5 + xs);
        const double ket = 2 * nE * nm + 2 * np2(Lf + d) * np2(Le) + nFp * (2 * (Le + 1) + 3 + xs);
        return n * (20 + 3 * 5 * na * nm + bra + ket + (d == 2 ? 20 : 0));
    }
    double per_root = 20 + 3 * 5 * vrr + 3 * 2 * hrr;
    if (mode == CG_MODE_IP1) per_root += 3 * 3 * (double)L.G / L.dI * (L.dI - 1) + 9.0 * L.nf;
    else if (mode == CG_MODE_IPIP1)
        per_root += 3 * 3 * (double)L.G / L.dI * (2 * L.dI - 3) + 18.0 * L.nf;
    else if (mode == CG_MODE_IP2) per_root += 3 * 3 * (double)L.G / L.dK * (L.dK - 1) + 9.0 * L.nf;
    else if (mode == CG_MODE_GRAD || mode == CG_MODE_GRADA) {
        double nT = (double)(li + 1) * (lj + 1) * (lk + 1) * (ll + 1);
        per_root += 9.0 * L.nf + 3 * nT * (mode == CG_MODE_GRADA ? 20 : 12);
    } else per_root += 3.0 * L.nf;
    return n * per_root;
}

}  // namespace

/* Contraction-first tables of one int2e / int3c2e class in kernel order (li >= lj, lk >= ll;
 * na = li + lj + 1 is the row length of the VRR arrays): the stage-3 groups, the permutations
 * from the transfer's Cartesian order to the accumulator rows/columns, and the transfer's buffer
 * size.  Layout described with CGEriClass. */
static int build_eri_class_tables(CINTGPUPlan *P, int li, int lj, int lk, int ll, bool bra);

/* The tables of a class depend on (li, lj, lk, ll, bra) alone: built once per process (the round
 * cutting is a dynamic program over the groups) and appended to each plan that uses the class. */
namespace {
struct EriTables {
    CGEriClass c;
    std::vector<CGEriGroup> groups;
    std::vector<int> perm, prog, rounds;
};
std::mutex g_eri_cache_mu;
std::unordered_map<int, std::shared_ptr<const EriTables>> g_eri_cache;
}  // namespace

static int build_eri_class(CINTGPUPlan *P, int li, int lj, int lk, int ll, bool bra)
{
    const int key = (((li * 16 + lj) * 16 + lk) * 16 + ll) * 2 + (bra ? 1 : 0);
    std::shared_ptr<const EriTables> t;
    {
        std::lock_guard<std::mutex> lk_(g_eri_cache_mu);
        auto it = g_eri_cache.find(key);
        if (it != g_eri_cache.end()) t = it->second;
    }
    if (!t) {
        CINTGPUPlan tmp;
        build_eri_class_tables(&tmp, li, lj, lk, ll, bra);
        auto e = std::make_shared<EriTables>();
        e->c = tmp.eclass[0];
        e->groups = tmp.egroup;
        e->perm = tmp.eperm;
        e->prog = tmp.hprog;
        e->rounds = tmp.eround;
        std::lock_guard<std::mutex> lk_(g_eri_cache_mu);
        t = g_eri_cache.emplace(key, e).first->second;
    }
    CGEriClass c = t->c;
    c.group_off = (int)P->egroup.size();
    c.perm_off = (int)P->eperm.size();
    c.hprog_off = (int)P->hprog.size();
    c.round_off = (int)P->eround.size();
    P->egroup.insert(P->egroup.end(), t->groups.begin(), t->groups.end());
    P->eperm.insert(P->eperm.end(), t->perm.begin(), t->perm.end());
    P->hprog.insert(P->hprog.end(), t->prog.begin(), t->prog.end());
    P->eround.insert(P->eround.end(), t->rounds.begin(), t->rounds.end());
    P->hrr_max = std::max(P->hrr_max, c.hrr_need);
    P->nef_max = std::max(P->nef_max, c.nE * c.nF);
    P->eclass.push_back(c);
    return (int)P->eclass.size() - 1;
}

static int build_eri_class_tables(CINTGPUPlan *P, int li, int lj, int lk, int ll, bool bra)
{
    struct Side {
        std::vector<int> x, y, z0, nz, base, pidx;
        int n = 0, lmax = 0;
    };
    auto side = [](int l0, int l1) {
        Side S;
        S.lmax = l0 + l1;
        S.pidx.assign((S.lmax + 1) * (S.lmax + 1), -1);
        for (int x = 0; x <= S.lmax; x++)
            for (int y = 0; x + y <= S.lmax; y++) {
                int z0 = std::max(0, l0 - x - y);
                S.pidx[x * (S.lmax + 1) + y] = (int)S.x.size();
                S.x.push_back(x); S.y.push_back(y); S.z0.push_back(z0);
                S.nz.push_back(S.lmax - x - y - z0 + 1);
                S.base.push_back(S.n);
                S.n += S.lmax - x - y - z0 + 1;
            }
        return S;
    };
    /* bra classes: one E entry per Cartesian pair (i, j), row i nfj + j, axis offsets
     * i + dI j in the per-term arrays g(i, j, f) (dI = li + 1); z powers fixed (one member) */
    auto bra_side = [&]() {
        Side S;
        S.lmax = li + lj;
        const int dI = li + 1;
        for (int ix = li; ix >= 0; ix--)
            for (int iy = li - ix; iy >= 0; iy--)
                for (int jx = lj; jx >= 0; jx--)
                    for (int jy = lj - jx; jy >= 0; jy--) {
                        S.x.push_back(ix + dI * jx);
                        S.y.push_back(iy + dI * jy);
                        S.z0.push_back((li - ix - iy) + dI * (lj - jx - jy));
                        S.nz.push_back(1);
                        S.base.push_back(S.n);
                        S.n++;
                    }
        return S;
    };
    const Side E = bra ? bra_side() : side(li, lj), F = side(lk, ll);
    /* stride of f in the per-term axis arrays */
    const int na = bra ? (li + 1) * (lj + 1) : li + lj + 1;
    CGEriClass c;
    c.nE = E.n;
    c.nF = F.n;
    c.group_off = (int)P->egroup.size();
    std::vector<CGEriGroup> g;
    for (size_t p = 0; p < E.x.size(); p++)
        for (size_t q = 0; q < F.x.size(); q++) {
            CGEriGroup e;
            e.oxy = (E.x[p] + na * F.x[q]) | ((E.y[p] + na * F.y[q]) << 16);
            e.oz = E.z0[p] + na * F.z0[q];
            e.acc = E.base[p] * F.n + F.base[q];
            e.mn = E.nz[p] | (F.nz[q] << 8);
            g.push_back(e);
        }
    /* Rounds: the kernel runs a class's groups in rounds of <= 32 (one per lane), each round
     * dispatched on its member box (largest nez x largest nfz).  A round costs 32 (box + 1) FP64
     * slots per term whatever its lanes need, so the groups are ordered by shape and cut into
     * rounds by dynamic programming over that order (two orders tried, the cheaper kept). */
    auto nez_of = [](const CGEriGroup &x) { return x.mn & 0xff; };
    auto nfz_of = [](const CGEriGroup &x) { return (x.mn >> 8) & 0xff; };
    auto cut = [&](const std::vector<CGEriGroup> &v, std::vector<std::pair<int, int>> *rounds) {
        const int n = (int)v.size();
        std::vector<double> best(n + 1, 1e300);
        std::vector<int> from(n + 1, 0);
        best[0] = 0;
        for (int i = 1; i <= n; i++) {
            int ma = 0, mb = 0;
            for (int j = i - 1; j >= std::max(0, i - 32); j--) {
                ma = std::max(ma, nez_of(v[j]));
                mb = std::max(mb, nfz_of(v[j]));
                double c = best[j] + 32.0 * (ma * mb + 1);
                if (c < best[i]) { best[i] = c; from[i] = j; }
            }
        }
        rounds->clear();
        for (int i = n; i > 0; i = from[i]) rounds->push_back({from[i], i - from[i]});
        std::reverse(rounds->begin(), rounds->end());
        return best[n];
    };
    std::vector<CGEriGroup> g2 = g;
    std::stable_sort(g.begin(), g.end(), [&](const CGEriGroup &a, const CGEriGroup &b) {
        if (nez_of(a) != nez_of(b)) return nez_of(a) > nez_of(b);
        return nfz_of(a) > nfz_of(b);
    });
    std::stable_sort(g2.begin(), g2.end(), [&](const CGEriGroup &a, const CGEriGroup &b) {
        if (nfz_of(a) != nfz_of(b)) return nfz_of(a) > nfz_of(b);
        return nez_of(a) > nez_of(b);
    });
    std::vector<std::pair<int, int>> r1, r2;
    if (cut(g2, &r2) < cut(g, &r1)) { g.swap(g2); r1.swap(r2); }
    P->egroup.insert(P->egroup.end(), g.begin(), g.end());
    c.round_off = (int)P->eround.size();
    c.nround = (int)r1.size();
    for (const auto &r : r1) {
        int ma = 1, mb = 1;
        for (int k = r.first; k < r.first + r.second; k++) {
            ma = std::max(ma, nez_of(g[k]));
            mb = std::max(mb, nfz_of(g[k]));
        }
        const int box = (ma <= 4 && mb <= 4) ? (ma - 1) + 4 * (mb - 1) : 0xff;
        P->eround.push_back(r.first | (r.second << 16) | (box << 24));
    }
    c.ngroup = (int)g.size();
    c.split = 0;
    if (c.ngroup <= 32) {
        int sp = 1;
        while (2 * sp * c.ngroup <= 32) sp *= 2;
        c.split = sp;
    }
    c.perm_off = (int)P->eperm.size();
    auto perm = [&](const Side &S, int l0) {
        for (int l = l0; l <= S.lmax; l++)
            for (int x = l; x >= 0; x--)
                for (int y = l - x; y >= 0; y--) {
                    int p = S.pidx[x * (S.lmax + 1) + y];
                    P->eperm.push_back(S.base[p] + (l - x - y) - S.z0[p]);
                }
    };
    if (bra)   /* rows are already in the transfer's order (i nfj + j) */
        for (int e = 0; e < c.nE; e++) P->eperm.push_back(e);
    else
        perm(E, li);
    perm(F, lk);
    auto below = [](int l) { return l * (l + 1) * (l + 2) / 6; };
    int need = std::max(c.nE * c.nF, ncart_l(li) * ncart_l(lj) * ncart_l(lk) * ncart_l(ll));
    for (int b = 1; b <= (bra ? 0 : lj); b++)
        need = std::max(need, (below(li + lj - b + 1) - below(li)) * ncart_l(b) * c.nF);
    for (int d = 1; d <= ll; d++)
        need = std::max(need, ncart_l(li) * ncart_l(lj) * (below(lk + ll - d + 1) - below(lk)) * ncart_l(d));
    c.hrr_need = need;
    c.maxab = (bra ? 1 : lj + 1) | ((ll + 1) << 8);
    /* transfer program: per bra level b = 1..lj, nrows then (hi, lo, axis) per row (e, jb):
     * row = e_hi(e + 1_ax, jb - 1_ax), lo = (e, jb - 1_ax), ax = lowest non-zero axis of jb;
     * per ket level d = 1..ll, nent, in_stride, out_stride, then (hi, lo, axis) per (f, ld) */
    c.hprog_off = (int)P->hprog.size();
    c.bra = bra ? 1 : 0;
    auto cidx = [](int l, int x, int y) { int r = l - x; return r * (r + 1) / 2 + (r - y); };
    auto comps = [](int l) {
        std::vector<std::array<int, 3>> v;
        for (int x = l; x >= 0; x--)
            for (int y = l - x; y >= 0; y--) v.push_back({x, y, l - x - y});
        return v;
    };
    for (int b = 1; b <= (bra ? 0 : lj); b++) {
        const int ncb1 = ncart_l(b - 1);
        const auto jb_list = comps(b);
        int nrows = (below(li + lj - b + 1) - below(li)) * ncart_l(b);
        P->hprog.push_back(nrows);
        for (int el = li; el <= li + lj - b; el++)
            for (const auto &e : comps(el))
                for (const auto &j : jb_list) {
                    const int ax = j[0] > 0 ? 0 : (j[1] > 0 ? 1 : 2);
                    const int dx = ax == 0, dy = ax == 1;
                    const int jp = cidx(b - 1, j[0] - dx, j[1] - dy);
                    const int ei = below(el) - below(li) + cidx(el, e[0], e[1]);
                    const int eu = below(el + 1) - below(li) + cidx(el + 1, e[0] + dx, e[1] + dy);
                    P->hprog.push_back(eu * ncb1 + jp);
                    P->hprog.push_back(ei * ncb1 + jp);
                    P->hprog.push_back(ax);
                }
    }
    int nFprev = c.nF;
    for (int d = 1; d <= ll; d++) {
        const int ncd = ncart_l(d), ncd1 = ncart_l(d - 1);
        const int nFp = below(lk + ll - d + 1) - below(lk);
        P->hprog.push_back(nFp * ncd);
        P->hprog.push_back(nFprev * ncd1);
        P->hprog.push_back(nFp * ncd);
        const auto ld_list = comps(d);
        for (int fl = lk; fl <= lk + ll - d; fl++)
            for (const auto &f : comps(fl))
                for (const auto &l : ld_list) {
                    const int ax = l[0] > 0 ? 0 : (l[1] > 0 ? 1 : 2);
                    const int dx = ax == 0, dy = ax == 1;
                    const int lp = cidx(d - 1, l[0] - dx, l[1] - dy);
                    const int fi = below(fl) - below(lk) + cidx(fl, f[0], f[1]);
                    const int fu = below(fl + 1) - below(lk) + cidx(fl + 1, f[0] + dx, f[1] + dy);
                    P->hprog.push_back(fu * ncd1 + lp);
                    P->hprog.push_back(fi * ncd1 + lp);
                    P->hprog.push_back(ax);
                }
        nFprev = nFp;
    }
    P->hrr_max = std::max(P->hrr_max, need);
    P->nef_max = std::max(P->nef_max, c.nE * c.nF);
    P->eclass.push_back(c);
    return (int)P->eclass.size() - 1;
}

/* Adjoint iteration tables of one class (kernel order li, lj, lk, ll): for every axis a and a-axis
 * power tuple u, the Cartesian components sharing u, as (partner g offsets, component index),
 * in chunks of <= 16 sorted longest first.  See rys_grad.cu. */
static int build_grad_class(CINTGPUPlan *P, int li, int lj, int lk, int ll)
{
    CGLayout L;
    cg_layout(li, lj, lk, ll, P->mode, CG_WS_MAX, &L);
    const int l[4] = {li, lj, lk, ll};
    const int nfc[4] = {ncart_l(li), ncart_l(lj), ncart_l(lk), ncart_l(ll)};
    auto cidx = [](int lq, int lx, int ly) { int r = lq - lx; return r * (r + 1) / 2 + (r - ly); };
    struct Ch { int axis_u, ent, len, ou, p0, p1, p2; };
    std::vector<Ch> list;
    for (int a = 0; a < 3; a++) {
        const int b = a == 2 ? 0 : a + 1, c = 3 - a - b;
        int u = 0;
        for (int p3 = 0; p3 <= l[3]; p3++)
        for (int p2 = 0; p2 <= l[2]; p2++)
        for (int p1 = 0; p1 <= l[1]; p1++)
        for (int p0 = 0; p0 <= l[0]; p0++) {
            u = ((p3 * (l[2] + 1) + p2) * (l[1] + 1) + p1) * (l[0] + 1) + p0;
            const int p[4] = {p0, p1, p2, p3};
            int start = (int)P->gent.size();
            for (int b3 = 0; b3 <= l[3] - p[3]; b3++)
            for (int b2 = 0; b2 <= l[2] - p[2]; b2++)
            for (int b1 = 0; b1 <= l[1] - p[1]; b1++)
            for (int b0 = 0; b0 <= l[0] - p[0]; b0++) {
                const int bb[4] = {b0, b1, b2, b3};
                int cc[4], pw[3][4];
                for (int q = 0; q < 4; q++) {
                    cc[q] = l[q] - p[q] - bb[q];
                    pw[a][q] = p[q]; pw[b][q] = bb[q]; pw[c][q] = cc[q];
                }
                int ob = ((bb[0] * L.dJ + bb[1]) * L.dK + bb[2]) * L.dL + bb[3];
                int oc = ((cc[0] * L.dJ + cc[1]) * L.dK + cc[2]) * L.dL + cc[3];
                int ci[4];
                for (int q = 0; q < 4; q++) ci[q] = cidx(l[q], pw[0][q], pw[1][q]);
                CGGradEnt e;
                e.ob_oc = ob | (oc << 16);
                e.c = ((ci[0] * nfc[1] + ci[1]) * nfc[2] + ci[2]) * nfc[3] + ci[3];
                P->gent.push_back(e);
            }
            int total = (int)P->gent.size() - start;
            int ou = ((p0 * L.dJ + p1) * L.dK + p2) * L.dL + p3;
            for (int o = 0; o < total; o += 16)
                list.push_back({a | (u << 2), start + o, std::min(16, total - o), ou, p0, p1, p2});
        }
    }
    std::stable_sort(list.begin(), list.end(), [](const Ch &x, const Ch &y) { return x.len > y.len; });
    CGGradClass gc;
    gc.chunk_off = (int)P->gchunk.size();
    gc.nchunk = (int)list.size();
    gc.pad0 = gc.pad1 = 0;
    for (const Ch &x : list) {
        CGGradChunk g;
        g.axis_u = x.axis_u; g.ent = x.ent; g.len = x.len; g.ou = x.ou; g.pad = 0;
        g.om[0] = x.p0 ? x.ou - L.dJ * L.dK * L.dL : x.ou;
        g.om[1] = x.p1 ? x.ou - L.dK * L.dL : x.ou;
        g.om[2] = x.p2 ? x.ou - L.dL : x.ou;
        g.p[0] = x.p0; g.p[1] = x.p1; g.p[2] = x.p2;
        P->gchunk.push_back(g);
    }
    P->gclass.push_back(gc);
    return (int)P->gclass.size() - 1;
}

static void free_plan_device(CINTGPUPlan *p)
{
    if (p->owns_dbuf && p->dbuf) cudaFree(p->dbuf);
    p->dbuf = nullptr;
    if (p->ev_fork) cudaEventDestroy(p->ev_fork);
    if (p->ev_join) cudaEventDestroy(p->ev_join);
    if (p->ev_t0) cudaEventDestroy(p->ev_t0);
    if (p->ev_t1) cudaEventDestroy(p->ev_t1);
    p->ev_t0 = p->ev_t1 = nullptr;
    if (p->side) cudaStreamDestroy(p->side);
    p->ev_fork = p->ev_join = nullptr;
    p->side = nullptr;
}

/* Where the horizontal transfers run (kernel order, so lj <= li and ll <= lk).  Transferring a
 * contracted 3D block multiplies the three axes' rounding amplifications, where libcint's
 * per-axis transfers of each primitive's 2D integrals only add them.  Measured against a
 * long-double evaluation on the c1 classes: contraction first leaves up to 6.8e-9 relative error
 * on uncancelled Cartesian elements of f-f transfers and ~5e-12 of the block scale on (fd|dd)
 * (libcint: 1.1e-10 and 7e-15); with lj or ll >= 4 it even leaves the 1e-12 absolute bar
 * ((ih|ih): 1.2e-12).  So:
 *   ll >= prim_l (default 4)          both transfers per primitive (CG_MODE_ERIP);
 *   lj >= bra_l (default 2), li + lj >= bra_lsum (default 5), ll < prim_l
 *                                     the bra transfer per term, the ket transfer (ll <= 3:
 *                                     (ff|ff) keeps 8.8e-12 relative on uncancelled Cartesian
 *                                     elements, 5% faster than per primitive) after contraction
 *                                     (CG_MODE_ERIB);
 *   otherwise                         both transfers after contraction (contraction first):
 *                                     (dd| included, which stays within 1e-11 relative of the
 *                                     long-double evaluation on 100 c1 quartets per class where
 *                                     (fd| and (gd| reach 2e-10 and 4.5e-10 that way.
 * A class whose per-term arrays do not fit the largest per-warp shared memory falls back to the
 * next route that fits ((ii|ii)-type classes: contraction first). */
static bool erip_fits(const int *l)
{
    CGLayout L;
    cg_layout(l[0], l[1], l[2], l[3], CG_MODE_ERIP, CG_WS_MAX, &L);
    return L.T >= 1 && L.G < 2048;
}
static bool bra_term(const CINTGPUPlan *P, const int *l)
{
    if (P->mode != CG_MODE_ERI || l[1] < P->bra_l || l[0] + l[1] < P->bra_lsum || l[3] >= P->prim_l)
        return false;
    /* stage-3 rounds address groups with 16 bits */
    if (ncart_l(l[0]) * ncart_l(l[1]) * ncart_l(l[2] + l[3]) >= 65536) return false;
    CGLayout L;
    cg_layout(l[0], l[1], l[2], l[3], CG_MODE_ERIB, CG_WS_MAX, &L);
    return L.T >= 1;
}
/* adjoint kernel of a plan */
static int grad_kernel_mode(const CINTGPUPlan *P)
{
    if (!P->gradj) return P->mode;
    return P->mode == CG_MODE_GRADA ? CG_MODE_GRADAJ : CG_MODE_GRADJ;
}
/* kernel (layout) mode of one class */
static int class_mode(const CINTGPUPlan *P, const int *l)
{
    if (P->gradj) return P->mode == CG_MODE_GRADA ? CG_MODE_GRADAJ : CG_MODE_GRADJ;
    return bra_term(P, l) ? CG_MODE_ERIB : P->mode;
}
static bool per_primitive(const CINTGPUPlan *P, const int *l)
{
    if (P->mode != CG_MODE_ERI || (l[1] < P->prim_l && l[3] < P->prim_l)) return false;
    if (bra_term(P, l)) return false;
    return erip_fits(l);
}

/* Build the host images. split_target: minimum number of compute tasks wanted (0 = no split). */
/* shell indices per item of an integral kind */
static int kind_shells(int kind)
{
    if (kind == CINTGPU_INT3C2E_SPH || kind == CINTGPU_INT3C2E_CART || kind == CINTGPU_INT3C2E_IP1_SPH
        || kind == CINTGPU_INT3C2E_IP1_CART || kind == CINTGPU_INT3C2E_IP2_SPH
        || kind == CINTGPU_INT3C2E_IP2_CART) return 3;
    if (kind == CINTGPU_INT2C2E_SPH || kind == CINTGPU_INT2C2E_CART) return 2;
    return 4;
}

static bool kind_sph(int kind)
{
    return kind == CINTGPU_INT2E_SPH || kind == CINTGPU_INT2E_IP1_SPH || kind == CINTGPU_INT3C2E_SPH
        || kind == CINTGPU_INT2C2E_SPH || kind == CINTGPU_INT2E_IP2_SPH || kind == CINTGPU_INT2E_IPIP1_SPH
        || kind == CINTGPU_INT3C2E_IP1_SPH || kind == CINTGPU_INT3C2E_IP2_SPH;
}

static bool fused(const CINTGPUPlan *P);

static int build_plan(CINTGPUPlan *P, int kind, const int *shls, int64_t n, const int64_t *offsets,
                      const int *atm, int natm, const int *bas, int nbas, const double *env,
                      int64_t split_target, OptState *opt = nullptr)
{
    (void)nbas;
    P->kind = kind;
    if (const char *e = getenv("CINTGPU_PER_PRIMITIVE_L")) P->prim_l = std::max(0, atoi(e));
    if (const char *e = getenv("CINTGPU_BRA_TERM_L")) P->bra_l = std::max(0, atoi(e));
    switch (kind) {
    case CINTGPU_INT2E_SPH: P->mode = CG_MODE_ERI; P->sph = 1; P->three = 0; break;
    case CINTGPU_INT2E_CART: P->mode = CG_MODE_ERI; P->sph = 0; P->three = 0; break;
    case CINTGPU_INT2E_IP1_SPH: P->mode = CG_MODE_IP1; P->sph = 1; P->three = 0; break;
    case CINTGPU_INT2E_IP1_CART: P->mode = CG_MODE_IP1; P->sph = 0; P->three = 0; break;
    case CINTGPU_INT2E_IP2_SPH: P->mode = CG_MODE_IP2; P->sph = 1; P->three = 0; break;
    case CINTGPU_INT2E_IP2_CART: P->mode = CG_MODE_IP2; P->sph = 0; P->three = 0; break;
    case CINTGPU_INT2E_IPIP1_SPH: P->mode = CG_MODE_IPIP1; P->sph = 1; P->three = 0; break;
    case CINTGPU_INT2E_IPIP1_CART: P->mode = CG_MODE_IPIP1; P->sph = 0; P->three = 0; break;
    case CINTGPU_INT3C2E_IP1_SPH: P->mode = CG_MODE_IP1; P->sph = 1; P->three = 1; break;
    case CINTGPU_INT3C2E_IP1_CART: P->mode = CG_MODE_IP1; P->sph = 0; P->three = 1; break;
    case CINTGPU_INT3C2E_IP2_SPH: P->mode = CG_MODE_IP2; P->sph = 1; P->three = 1; break;
    case CINTGPU_INT3C2E_IP2_CART: P->mode = CG_MODE_IP2; P->sph = 0; P->three = 1; break;
    case CINTGPU_INT3C2E_SPH: P->mode = CG_MODE_ERI; P->sph = 1; P->three = 1; break;
    case CINTGPU_INT3C2E_CART: P->mode = CG_MODE_ERI; P->sph = 0; P->three = 1; break;
    case CINTGPU_INT2C2E_SPH: P->mode = CG_MODE_ERI; P->sph = 1; P->three = 1; P->two = 1; break;
    case CINTGPU_INT2C2E_CART: P->mode = CG_MODE_ERI; P->sph = 0; P->three = 1; P->two = 1; break;
    case CINTGPU_J_BUILD: P->mode = CG_MODE_ERI; P->sph = 0; P->three = 0; P->jmode = 1; break;
    case CINTGPU_K_BUILD: P->mode = CG_MODE_ERI; P->sph = 0; P->three = 0; P->jmode = 2; break;
    case CINTGPU_JK_BUILD: P->mode = CG_MODE_ERI; P->sph = 0; P->three = 0; P->jmode = 3; break;
    case CINTGPU_J_GRAD:
        P->mode = CG_MODE_GRAD; P->sph = 0; P->three = 0;
        /* CINTGPU_ADJOINT=component: the per-component adjoint kernel instead */
        {
            const char *e = getenv("CINTGPU_ADJOINT");
            P->gradj = !(e && strcmp(e, "component") == 0);
        }
        break;
    case CINTGPU_J_GRAD_EXP:
        P->mode = CG_MODE_GRADA; P->sph = 0; P->three = 0;
        {
            const char *e = getenv("CINTGPU_ADJOINT");
            P->gradj = !(e && strcmp(e, "component") == 0);
        }
        break;
    default: set_error("unknown integral kind %d", kind); return CINTGPU_ERR_ARG;
    }
    P->ncomp = CG_NCOMP(P->mode);
    /* env[PTR_RANGE_OMEGA] > 0: long-range Coulomb erf(omega r)/r (src/g2e.c:4477-4492), the same
     * screening as 1/r; < 0: short-range erfc(|omega| r)/r (src/g2e.c:4447-4476), kept as
     * -omega^2: the kernels evaluate 2n terms per primitive quartet (full minus long range) and
     * drop primitive quartets whose attenuated integral libcint neglects */
    if (!std::isfinite(env[PTR_RANGE_OMEGA])) {
        set_error("env[PTR_RANGE_OMEGA] = %g is not finite", env[PTR_RANGE_OMEGA]);
        return CINTGPU_ERR_ARG;
    }
    P->omega2 = (env[PTR_RANGE_OMEGA] < 0 ? -1.0 : 1.0) * env[PTR_RANGE_OMEGA] * env[PTR_RANGE_OMEGA];
    /* src/g2e.c:57-62 (+1), src/g3c2e.c:55-59 and src/g2c2e.c:44-48 (no +1) */
    if (env[PTR_EXPCUTOFF] == 0) P->expcutoff = 60;
    else P->expcutoff = std::max(40.0, env[PTR_EXPCUTOFF]) + (P->three ? 0 : 1);
    P->nitems = n;
    P->natm = natm;
    Builder B{P, atm, natm, bas, env, {}, {}, {}};
    const bool contracting = P->jmode || P->mode == CG_MODE_GRAD || P->mode == CG_MODE_GRADA;
    if (!contracting) B.opt = opt;   /* the cached pairs carry no AO / primitive offsets */
    std::vector<int> ao_loc, prim_loc;
    if (contracting) {
        ao_loc.resize(nbas + 1);
        prim_loc.resize(nbas + 1);
        ao_loc[0] = prim_loc[0] = 0;
        for (int i = 0; i < nbas; i++) {
            const int *b = bas + BAS_SLOTS * i;
            ao_loc[i + 1] = ao_loc[i] + ncart_l(b[ANG_OF]) * b[NCTR_OF];
            prim_loc[i + 1] = prim_loc[i] + b[NPRIM_OF];
        }
        P->nao_cart = ao_loc[nbas];
        P->nprim_tot = prim_loc[nbas];
        B.ao_loc = &ao_loc;
        B.prim_loc = &prim_loc;
    }
    const int nsh = kind_shells(kind);
    /* the derivative raises the l ceiling entering libcint's log_rr of the differentiated pair */
    const int dinc = P->mode == CG_MODE_IP1 ? 1 : (P->mode == CG_MODE_IPIP1 ? 2 : 0);
    const int dinc_k = P->mode == CG_MODE_IP2 ? 1 : 0;

    struct Pending { int pij, pkl, out; int64_t npq; int l[4]; int sym; };
    std::vector<Pending> pend;
    pend.reserve((size_t)n);            /* at least one entry per item (more with nctr > 1) */
    P->outs.reserve(P->outs.size() + (size_t)n);
    P->out_item.reserve(P->out_item.size() + (size_t)n);
    std::vector<char> finite_checked;   /* per shell index: data checked once per plan */
    int64_t next_off = 0;
    for (int64_t q = 0; q < n; q++) {
        const int *s = shls + nsh * q;
        ShellView sv[4];
        for (int a = 0; a < nsh; a++) {
            int rc = read_shell(s[a], atm, natm, bas, env, &sv[a]);
            if (rc) return rc;
            if (s[a] > PAIR_KEY_MAX_SHELL) { set_error("shell index %d above %d", s[a], PAIR_KEY_MAX_SHELL); return CINTGPU_ERR_ARG; }
            if ((size_t)s[a] >= finite_checked.size()) finite_checked.resize((size_t)s[a] + 1, 0);
            if (!finite_checked[s[a]]) {
                if ((rc = check_finite(s[a], sv[a]))) return rc;
                finite_checked[s[a]] = 1;
            }
            if (contracting && s[a] >= nbas) { set_error("shell %d outside nbas %d", s[a], nbas); return CINTGPU_ERR_ARG; }
            if (P->mode == CG_MODE_GRAD || P->mode == CG_MODE_GRADA) {
                if (sv[a].l > 4) { set_error("adjoint supports l <= 4 (shell %d has %d)", s[a], sv[a].l); return CINTGPU_ERR_UNSUPPORTED; }
                if (P->mode == CG_MODE_GRADA && sv[a].nprim > CG_GRAD_MAXPRIM) {
                    set_error("exponent adjoint supports nprim <= %d", CG_GRAD_MAXPRIM);
                    return CINTGPU_ERR_UNSUPPORTED;
                }
            }
        }
        /* int2c2e (i|k) runs as (i s0|k s0): request shells 0, 1 in kernel slots 0, 2 */
        if (P->two) { sv[2] = sv[1]; sv[1] = sv[0]; sv[1].l = 0; sv[1].nprim = 1; sv[1].nctr = 1; }
        if (P->three) { sv[3] = sv[2]; sv[3].l = 0; sv[3].nprim = 1; sv[3].nctr = 1; }
        auto unit = [&](int a) { return (a == 3 && P->three) || (a == 1 && P->two); };
        int d[4], nd[4];
        for (int a = 0; a < 4; a++) {
            d[a] = unit(a) ? 1 : (P->sph ? nsph_l(sv[a].l) : ncart_l(sv[a].l));
            nd[a] = d[a] * (unit(a) ? 1 : sv[a].nctr);
        }
        int64_t req_st[4] = {1, nd[0], (int64_t)nd[0] * nd[1], (int64_t)nd[0] * nd[1] * nd[2]};
        if (P->three) req_st[3] = 0;
        if (P->two) req_st[1] = 0;
        int64_t block = (int64_t)nd[0] * nd[1] * nd[2] * nd[3];
        int64_t base = offsets ? offsets[q] : next_off;
        next_off = std::max(next_off, base + block);
        /* kernel order: perm[k] = request index placed at kernel slot k.  Inside a pair the
         * larger l comes first (it is the recurrence base); for equal l the shell whose most
         * diffuse exponent is larger: the product densities then sit near the base centre, so
         * the transfer (i, j+1) = (i+1, j) + AB (i, j) does not build (i j| from large moments
         * about a distant centre (a distant, exponent-asymmetric f-f pair loses ~3e-7 of its
         * largest diagonal element with the base on the diffuse shell, libcint included). */
        auto amin = [](const ShellView &v) { return *std::min_element(v.ex, v.ex + v.nprim); };
        auto first = [&](int a, int b) {   /* shell a goes before shell b */
            return sv[a].l > sv[b].l || (sv[a].l == sv[b].l && amin(sv[a]) >= amin(sv[b]));
        };
        int perm[4] = {0, 1, 2, 3};
        if (!CG_IS_IP(P->mode)) {   /* the nabla's shell keeps its slot */
            if (P->two ? sv[0].l < sv[1].l : !first(0, 1)) std::swap(perm[0], perm[1]);
            if (!P->three) {
                if (!first(2, 3)) std::swap(perm[2], perm[3]);
                int lij = sv[perm[0]].l * 16 + sv[perm[1]].l, lkl = sv[perm[2]].l * 16 + sv[perm[3]].l;
                if (lij < lkl) { std::swap(perm[0], perm[2]); std::swap(perm[1], perm[3]); }
            }
        }
        const ShellView *kv[4] = {&sv[perm[0]], &sv[perm[1]], &sv[perm[2]], &sv[perm[3]]};
        int ksh[4];
        for (int k = 0; k < 4; k++) ksh[k] = unit(k) ? -1 : s[P->two ? perm[k] / 2 : perm[k]];
        /* permutation flags of the unique quartet, in kernel order (the J epilogue weights the
         * kernel's bra and ket blocks with them) */
        int qsym = 0;
        if (!P->three) {
            int b0 = std::min(ksh[0], ksh[1]), b1 = std::max(ksh[0], ksh[1]);
            int k0 = std::min(ksh[2], ksh[3]), k1 = std::max(ksh[2], ksh[3]);
            qsym = (ksh[0] != ksh[1] ? 1 : 0) | (ksh[2] != ksh[3] ? 2 : 0)
                 | ((b0 != k0 || b1 != k1) ? 4 : 0);
        }
        int kl_[4] = {kv[0]->l, kv[1]->l, kv[2]->l, kv[3]->l};
        int nct[4] = {kv[0]->nctr, kv[1]->nctr, kv[2]->nctr, P->three ? 1 : kv[3]->nctr};
        for (int c3 = 0; c3 < nct[3]; c3++)
        for (int c2 = 0; c2 < nct[2]; c2++)
        for (int c1 = 0; c1 < nct[1]; c1++)
        for (int c0 = 0; c0 < nct[0]; c0++) {
            int cc[4] = {c0, c1, c2, c3};
            int pij = P->two ? B.single(ksh[0], *kv[0], c0)
                             : B.pair(ksh[0], *kv[0], c0, ksh[1], *kv[1], c1, kl_[0] + dinc + kl_[1]);
            int pkl = P->three ? B.single(ksh[2], *kv[2], c2)
                               : B.pair(ksh[2], *kv[2], c2, ksh[3], *kv[3], c3, kl_[2] + dinc_k + kl_[3]);
            CGOutTask o;
            memset(&o, 0, sizeof(o));
            o.out_off = base;
            for (int k = 0; k < 4; k++) {
                o.l[k] = kl_[k];
                o.st[k] = (int)req_st[perm[k]];
                o.out_off += (int64_t)cc[k] * d[perm[k]] * req_st[perm[k]];
            }
            o.flags = P->sph ? 1 : 0;
            o.nparts = 0;
            int out_id = (int)P->outs.size();
            P->outs.push_back(o);
            P->out_item.push_back((int)q);
            int nf = ncart_l(kl_[0]) * ncart_l(kl_[1]) * ncart_l(kl_[2]) * ncart_l(kl_[3]);
            P->max_nf = std::max(P->max_nf, nf);
            if (B.pair_empty[pij] || B.pair_empty[pkl]) continue;
            const CGPair &a = P->pairs[pij], &b = P->pairs[pkl];
            Pending pe{pij, pkl, out_id, (int64_t)a.npa * a.npb * b.npa * b.npb,
                       {kl_[0], kl_[1], kl_[2], kl_[3]}, qsym};
            pend.push_back(pe);
        }
    }
    P->out_size = next_off;
    /* Screening on the host with libcint's rule and loop order (src/cint2e.c:400-425: kl outer,
     * ij inner; skip kl if cce_kl > cutoff, skip ij if cce_ij > cutoff - cce_kl): the kernels get
     * the surviving primitive quartets as a list, so work can be sliced evenly. */
    struct Work { int pe; int64_t off, n; double cost_pq; };
    std::vector<Work> work;
    work.reserve(pend.size());
    /* per-class constants: classes ((li 8 + lj) 8 + lk) 8 + ll (l <= 7 with derivatives) map to
     * dense slots, so a plan of one quartet does not initialise tables for all 4096 */
    std::vector<int16_t> cls_slot(8 * 8 * 8 * 8, -1);
    std::vector<double> cls_cost, cls_ref;
    std::vector<int> cls_group;
    std::vector<CGLayout> cls_layout;
    auto slot_of = [&](int ck) -> int {
        if (cls_slot[ck] < 0) {
            cls_slot[ck] = (int16_t)cls_cost.size();
            cls_cost.push_back(-1.0);
            cls_ref.push_back(0.0);
            cls_group.push_back(-1);
            cls_layout.emplace_back();
        }
        return cls_slot[ck];
    };
    /* largest screening value of each pair's primitive pairs (NaN counts as +inf): when it is
     * within a ket primitive's limit every bra primitive pair survives and the test is skipped */
    std::vector<double> cce_max(P->pairs.size());
    for (size_t p = 0; p < P->pairs.size(); p++) {
        const CGPair &q = P->pairs[p];
        double mx = -INFINITY;
        for (int i = 0; i < q.npa * q.npb; i++) {
            const double c = P->prims[q.prim_off + i].cce;
            mx = std::max(mx, std::isnan(c) ? INFINITY : c);
        }
        cce_max[p] = mx;
    }
    /* survivors of one pending quartet in libcint's order (kl outer, ij inner), written to dst
     * unless it is null; returns their count */
    auto screen = [&](const Pending &pe, int *dst) -> int64_t {
        const CGPair &a = P->pairs[pe.pij], &b = P->pairs[pe.pkl];
        const CGPrimPair *pa = &P->prims[a.prim_off], *pb = &P->prims[b.prim_off];
        const int nij = a.npa * a.npb, nkl = b.npa * b.npb;
        const double amax = cce_max[pe.pij];
        int64_t m = 0;
        for (int kl = 0; kl < nkl; kl++) {
            const double ck = pb[kl].cce;
            if (ck > P->expcutoff) continue;
            const double lim = P->expcutoff - ck;
            if (!(amax > lim)) {
                if (dst)
                    for (int ij = 0; ij < nij; ij++) dst[m + ij] = kl * nij + ij;
                m += nij;
            } else {
                for (int ij = 0; ij < nij; ij++)
                    if (!(pa[ij].cce > lim)) {
                        if (dst) dst[m] = kl * nij + ij;
                        m++;
                    }
            }
        }
        return m;
    };
    /* count, prefix-sum, fill: on several threads for large lists (the positions, and so the
     * table, are the same as one thread's) */
    const size_t npend = pend.size();
    std::vector<int64_t> pos(npend + 1, 0);
    const int nthr = npend >= 50000 ? std::max(1, std::min(16, P->plan_threads)) : 1;
    auto over_pending = [&](const std::function<void(size_t, size_t)> &body) {
        if (nthr == 1) { body(0, npend); return; }
        std::vector<std::thread> th;
        for (int t = 0; t < nthr; t++) th.emplace_back(body, npend * t / nthr, npend * (t + 1) / nthr);
        for (std::thread &x : th) x.join();
    };
    over_pending([&](size_t b, size_t e) { for (size_t w = b; w < e; w++) pos[w + 1] = screen(pend[w], nullptr); });
    const int64_t base = (int64_t)P->pqlist.size();
    pos[0] = base;
    for (size_t w = 0; w < npend; w++) pos[w + 1] += pos[w];
    P->pqlist.resize((size_t)pos[npend]);
    over_pending([&](size_t b, size_t e) {
        for (size_t w = b; w < e; w++) screen(pend[w], P->pqlist.data() + pos[w]);
    });
    double fl = 0;
    for (size_t w = 0; w < npend; w++) {
        const Pending &pe = pend[w];
        const int64_t off = pos[w], n = pos[w + 1] - pos[w];
        const int ck = slot_of(((pe.l[0] * 8 + pe.l[1]) * 8 + pe.l[2]) * 8 + pe.l[3]);
        if (cls_cost[ck] < 0) {
            cls_cost[ck] = per_primitive(P, pe.l) ? flops_libcint_primq(pe.l[0], pe.l[1], pe.l[2], pe.l[3])
                         : flops_per_primq(pe.l[0], pe.l[1], pe.l[2], pe.l[3], class_mode(P, pe.l));
            if (P->omega2 < 0) cls_cost[ck] *= 2;   /* short range: full and long-range terms */
            cls_ref[ck] = P->mode == CG_MODE_ERI ? flops_libcint_primq(pe.l[0], pe.l[1], pe.l[2], pe.l[3]) : 0.0;
        }
        const double cpq = cls_cost[ck];
        fl += n * cpq;
        P->flops_ref += n * cls_ref[ck];
        if (n > 0) work.push_back({(int)w, off, n, cpq});
    }
    if (P->pqlist.size() > (size_t)INT32_MAX) { set_error("too many primitive quartets in one plan"); return CINTGPU_ERR_ARG; }
    P->flops = fl;
    P->prim_quartets = (int64_t)P->pqlist.size();
    /* slices: no task above ~1/32 of a warp's fair share (or 32 primitive quartets) */
    const double warps = (double)std::max(1, g_ctx.sm_count) * 8.0;
    double target = std::max(fl / (warps * 32.0), 2.0e5);
    if (split_target > 0) target = std::min(target, fl / (double)split_target);
    /* shared memory per warp of the regular group: 24 KB unless the plan's tuned value or
     * CINTGPU_WS_KB overrides it */
    int ws_small = CG_WS_SMALL;
    {
        int kb = P->ws_kb;
        if (!kb)
            if (const char *e = getenv("CINTGPU_WS_KB")) kb = atoi(e);
        if (kb >= 8 && kb <= 48) ws_small = kb * 1024 / 8;
    }
    /* per-primitive kernels run a pair's recurrences about its second centre when that shell is
     * the tighter one (larger smallest exponent): see g_axis */
    std::vector<signed char> swap_of(P->pairs.size(), -1);
    auto pair_swap = [&](int p) -> bool {
        if (swap_of[p] < 0) {
            const CGPair &q = P->pairs[p];
            double ma = INFINITY, mb = INFINITY;
            for (int t = 0; t < q.npa * q.npb; t++) {
                const CGPrimPair &pp = P->prims[q.prim_off + t];
                ma = std::min(ma, pp.aA);
                mb = std::min(mb, pp.a - pp.aA);
            }
            swap_of[p] = mb > ma ? 1 : 0;
        }
        return swap_of[p] == 1;
    };
    struct TaskCost { CGTask t; double cost; int group; };
    std::vector<TaskCost> tc;
    std::vector<signed char> turn_of(P->gradj ? P->prims.size() : 0, -1);
    std::vector<int> part_tmp;
    std::unordered_map<int, int> grad_cls, eri_cls;
    int64_t gpos = 0;
    for (const Work &w : work) {
        const Pending &pe = pend[w.pe];
        const int ck = slot_of(((pe.l[0] * 8 + pe.l[1]) * 8 + pe.l[2]) * 8 + pe.l[3]);
        if (cls_group[ck] < 0) {
            CGLayout Lc;
            const int lmode = class_mode(P, pe.l);
            cg_layout(pe.l[0], pe.l[1], pe.l[2], pe.l[3], lmode, ws_small, &Lc);
            cls_group[ck] = 0;
            if (per_primitive(P, pe.l)) {
                cg_layout(pe.l[0], pe.l[1], pe.l[2], pe.l[3], CG_MODE_ERIP, CG_WS_MAX, &Lc);
                cls_group[ck] = 2;
            } else if (Lc.T < 2 || std::find(P->wide.begin(), P->wide.end(),
                                             ((pe.l[0] * 8 + pe.l[1]) * 8 + pe.l[2]) * 8 + pe.l[3])
                                       != P->wide.end()) {
                cg_layout(pe.l[0], pe.l[1], pe.l[2], pe.l[3], lmode, CG_WS_MAX, &Lc);
                cls_group[ck] = 1;
            }
            cls_layout[ck] = Lc;
        }
        const CGLayout &L = cls_layout[ck];
        const int group = cls_group[ck];
        if (L.nroots > cg_rys_nmax() || L.T < 1 || L.G >= (group == 2 ? 2048 : 1024)) {
            set_error("class (%d %d|%d %d) beyond the kernel limits (nroots %d, max %d)",
                      pe.l[0], pe.l[1], pe.l[2], pe.l[3], L.nroots, cg_rys_nmax());
            return CINTGPU_ERR_UNSUPPORTED;
        }
        /* at least one batch of terms per slice, at least 4 primitive quartets; slices hold whole
         * batches (terms a multiple of T) so only a quartet's last slice has a partial batch */
        const int nt = L.nroots * (P->omega2 < 0 ? 2 : 1);   /* terms per primitive quartet */
        int64_t slice = std::max<int64_t>(std::max<int64_t>(4, (L.T + nt - 1) / nt),
                                          (int64_t)(target / w.cost_pq));
        {
            int a = L.T, b = nt;
            while (b) { int t = a % b; a = b; b = t; }
            const int64_t m = L.T / a;
            slice = (slice + m - 1) / m * m;
        }
        int nf = ncart_l(pe.l[0]) * ncart_l(pe.l[1]) * ncart_l(pe.l[2]) * ncart_l(pe.l[3]);
        int64_t slot = (int64_t)nf * P->ncomp;
        CGOutTask &o = P->outs[pe.out];
        o.cart_off = gpos;
        int cls = 0;
        const int key = ((pe.l[0] * 16 + pe.l[1]) * 16 + pe.l[2]) * 16 + pe.l[3];
        if (P->gradj) {
            cls = -1;   /* contraction-first adjoint: no per-class tables */
        } else if (P->mode == CG_MODE_GRAD || P->mode == CG_MODE_GRADA) {
            auto it = grad_cls.find(key);
            cls = it != grad_cls.end() ? it->second
                                       : (grad_cls[key] = build_grad_class(P, pe.l[0], pe.l[1], pe.l[2], pe.l[3]));
        } else if (group == 2) {
            cls = -1;   /* per primitive: Cartesian slots, no contraction-first tables */
        } else if (P->mode == CG_MODE_ERI) {
            auto it = eri_cls.find(key);
            cls = it != eri_cls.end() ? it->second
                                      : (eri_cls[key] = build_eri_class(P, pe.l[0], pe.l[1], pe.l[2], pe.l[3],
                                                                        bra_term(P, pe.l)));
            const CGEriClass &ec = P->eclass[cls];
            slot = (int64_t)ec.nE * ec.nF;
            o.flags |= 2;
            o.ecls = cls;
            for (int c = 0; c < 3; c++) {
                o.AB[c] = P->pairs[pe.pij].AB[c];
                o.CD[c] = P->pairs[pe.pkl].AB[c];
            }
        }
        /* the contraction-first adjoint expands a primitive pair's density about its first centre
         * with binomial terms up to (1 + 2 b / a)^lb times the result (a, b: the primitives'
         * exponents); where that exceeds 16 and the second centre would do better,
         * (1 + 2 a / b)^la, the pair is seen from the second centre (bits 3/4): the quartet's
         * primitive quartets are grouped by the two choices, each group sliced into its own
         * tasks */
        int64_t gbeg[5] = {0, w.n, w.n, w.n, w.n};
        if (P->gradj) {
            const CGPair &bp = P->pairs[pe.pij], &kp = P->pairs[pe.pkl];
            const int nij = bp.npa * bp.npb;
            auto turn = [&](const CGPair &pr, int i) {   /* cached per primitive pair */
                signed char &t = turn_of[pr.prim_off + i];
                if (t < 0) {
                    const CGPrimPair &x = P->prims[pr.prim_off + i];
                    const double a = x.aA, b = x.a - x.aA;
                    const double k0 = pr.lb * std::log1p(2.0 * b / a), k1 = pr.la * std::log1p(2.0 * a / b);
                    t = k0 > std::log(16.0) && k1 < k0 ? 1 : 0;
                }
                return t == 1;
            };
            auto grp = [&](int q) {
                return (turn(bp, q % nij) ? 1 : 0) | (turn(kp, q / nij) ? 2 : 0);
            };
            int *beg = P->pqlist.data() + w.off;
            part_tmp.assign(beg, beg + w.n);
            const std::vector<int> &tmp = part_tmp;
            int64_t cnt[4] = {0, 0, 0, 0};
            for (int64_t i = 0; i < w.n; i++) cnt[grp(tmp[i])]++;
            gbeg[0] = 0;
            for (int g = 0; g < 4; g++) gbeg[g + 1] = gbeg[g] + cnt[g];
            int64_t pos[4] = {gbeg[0], gbeg[1], gbeg[2], gbeg[3]};
            for (int64_t i = 0; i < w.n; i++) beg[pos[grp(tmp[i])]++] = tmp[i];
        }
        /* a quartet of one slice in a plan that transforms in the integral kernel accumulates
         * in the running warp's own slot (reused, so it stays in L2), not in one of its own */
        const bool own = P->fuse_out && P->mode == CG_MODE_ERI && !P->jmode && !P->gradj
                      && group != 2 && w.n <= slice;
        for (int g = 0; g < 4; g++)
        for (int64_t a0 = gbeg[g]; a0 < gbeg[g + 1]; a0 += slice) {
            TaskCost x;
            x.t.pij = pe.pij; x.t.pkl = pe.pkl;
            x.t.pq_off = (int)(w.off + a0);
            x.t.npq = (int)std::min<int64_t>(slice, gbeg[g + 1] - a0);
            x.t.cart_off = own ? 0 : gpos;
            x.t.out = pe.out;
            x.t.sym = pe.sym;
            if (group == 2 || CG_IS_IP(P->mode))   /* per-primitive recurrences: base choice */
                x.t.sym |= (pair_swap(pe.pij) ? 8 : 0) | (pair_swap(pe.pkl) ? 16 : 0);
            if (P->gradj) x.t.sym |= g << 3;
            x.t.cls = cls;
            x.t.own_slot = own ? 1 : 0;
            x.cost = x.t.npq * w.cost_pq;
            x.group = group;
            tc.push_back(x);
            o.nparts++;
            if (own) P->own_slots = true;
            else gpos += slot;
        }
    }
    /* longest tasks first within each launch (LPT order for the dynamic work counter): a stable
     * counting sort on the cost's logarithm (256 buckets per factor of two, so costs within 0.3 %
     * share a bucket and keep their creation order), group by group */
    constexpr int NB = 1 << 14;
    double cmax = 0.0;
    for (const TaskCost &x : tc) cmax = std::max(cmax, x.cost);
    std::vector<int> bkt(tc.size());
    std::vector<int64_t> cnt(3 * (size_t)NB + 1, 0);
    for (size_t i = 0; i < tc.size(); i++) {
        const double c = tc[i].cost;
        int b = NB - 1;
        if (c > 0 && cmax > 0) b = std::min(NB - 1, std::max(0, (int)(std::log2(cmax / c) * 256.0)));
        bkt[i] = tc[i].group * NB + b;
        cnt[bkt[i] + 1]++;
    }
    for (size_t k = 1; k < cnt.size(); k++) cnt[k] += cnt[k - 1];
    const size_t tbase = P->tasks.size();
    P->tasks.resize(tbase + tc.size());
    for (size_t i = 0; i < tc.size(); i++) P->tasks[tbase + cnt[bkt[i]]++] = tc[i].t;
    int64_t gstart = (int64_t)tbase;
    for (int g = 0; g < 3; g++) {
        int64_t ng = 0;
        for (const TaskCost &x : tc) ng += x.group == g;
        P->groups[g].task0 = (int)gstart;
        gstart += ng;
        P->groups[g].ntasks = (int)ng;
        P->groups[g].ws = g == 0 ? ws_small : CG_WS_MAX;
        P->groups[g].blocks_per_sm = (P->mode == CG_MODE_GRAD || P->mode == CG_MODE_GRADA)
                                         ? cg_grad_blocks_per_sm(grad_kernel_mode(P), P->groups[g].ws)
                                         : cg_blocks_per_sm(g == 2 ? CG_MODE_ERIP : P->mode, P->groups[g].ws);
        P->groups[g].nblocks = std::min(std::max(1, g_ctx.sm_count) * P->groups[g].blocks_per_sm,
                                        std::max(1, (P->groups[g].ntasks + 3) / 4));
    }
    /* own slots need the fused transform and one slot of the largest class per warp; where
     * either is missing (or the slots would pass 256 MB), those tasks get slots of their own */
    if (P->own_slots) {
        const int64_t warps = 4 * (int64_t)(P->groups[0].nblocks + P->groups[1].nblocks + P->groups[2].nblocks);
        if (!fused(P) || (double)warps * P->nef_max * 8.0 > 256.0 * (1 << 20)) {
            for (CGTask &t : P->tasks)
                if (t.own_slot) {
                    /* the quartet's only slice: its output reads the same slot */
                    const CGEriClass &ec = P->eclass[t.cls];
                    t.own_slot = 0;
                    t.cart_off = gpos;
                    P->outs[t.out].cart_off = gpos;
                    gpos += (int64_t)ec.nE * ec.nF;
                }
            P->own_slots = false;
        }
    }
    P->gctr_size = std::max<int64_t>(gpos, 1);
    P->empty_outs.clear();
    for (size_t q = 0; q < P->outs.size(); q++)
        if (P->outs[q].nparts == 0) P->empty_outs.push_back((int)q);
    return 0;
}

struct DevLayout {
    size_t pairs, prims, tasks, outs, pq, gcl, gch, gen, ecl, egr, epm, hpg, erd, emp, gctr, cnt, ne, scr, wscr;
    size_t done, oscr, wslot;
    int oscr_warps;
    int64_t wstride;
    int wwarps;
    size_t upload, total;
    int out_blocks;
    int64_t spw;
};

/* the integral kernel transforms and stores finished quartets itself (int2e, int3c2e, ip1) */
static bool fused(const CINTGPUPlan *P)
{
    if (!P->fuse_out || P->jmode || !(P->mode == CG_MODE_ERI || CG_IS_IP(P->mode))) return false;
    /* one transform slot per launched warp; classes with huge blocks (l = 5, 6) would need
     * gigabytes, so such plans transform in the separate kernel */
    const int64_t spw = 2 * (int64_t)P->max_nf + (P->eclass.empty() ? 0 : 2 * (int64_t)P->hrr_max);
    const int64_t warps = 4 * (int64_t)(P->groups[0].nblocks + P->groups[1].nblocks + P->groups[2].nblocks);
    return (double)spw * 8.0 * warps <= 512.0 * (1 << 20);
}

static DevLayout dev_layout(const CINTGPUPlan *P)
{
    auto al = [](size_t x) { return (x + 255) / 256 * 256; };
    DevLayout D;
    const bool fo = fused(P);
    /* the output kernel transforms every quartet, or (fused) only zero-fills the empty ones */
    const size_t nout_k = fo ? P->empty_outs.size() : P->outs.size();
    D.out_blocks = std::max(1, std::min<int>((int)((nout_k + 3) / 4), g_ctx.sm_count * 8));
    /* output scratch per warp: two cart->sph buffers, two transfer buffers (ERI mode) */
    D.spw = 2 * (int64_t)P->max_nf + (P->eclass.empty() ? 0 : 2 * (int64_t)P->hrr_max);
    D.pairs = al(sizeof(CGPair) * std::max<size_t>(P->pairs.size(), 1));
    D.prims = al(sizeof(CGPrimPair) * std::max<size_t>(P->prims.size(), 1));
    D.tasks = al(sizeof(CGTask) * std::max<size_t>(P->tasks.size(), 1));
    D.outs = al(sizeof(CGOutTask) * std::max<size_t>(P->outs.size(), 1));
    D.pq = al(sizeof(int) * std::max<size_t>(P->pqlist.size(), 1));
    D.gcl = al(sizeof(CGGradClass) * std::max<size_t>(P->gclass.size(), 1));
    D.gch = al(sizeof(CGGradChunk) * std::max<size_t>(P->gchunk.size(), 1));
    D.gen = al(sizeof(CGGradEnt) * std::max<size_t>(P->gent.size(), 1));
    D.ecl = al(sizeof(CGEriClass) * std::max<size_t>(P->eclass.size(), 1));
    D.egr = al(sizeof(CGEriGroup) * std::max<size_t>(P->egroup.size(), 1));
    D.epm = al(sizeof(int) * std::max<size_t>(P->eperm.size(), 1));
    D.hpg = al(sizeof(int) * std::max<size_t>(P->hprog.size(), 1));
    D.erd = al(sizeof(int) * std::max<size_t>(P->eround.size(), 1));
    D.emp = al(sizeof(int) * std::max<size_t>(P->empty_outs.size(), 1));
    D.done = al(sizeof(int) * std::max<size_t>(P->outs.size(), 1));
    D.oscr_warps = fo ? 4 * (P->groups[0].nblocks + P->groups[1].nblocks + P->groups[2].nblocks) : 0;
    D.oscr = fo ? al(sizeof(double) * (size_t)D.oscr_warps * D.spw) : 0;
    D.wslot = P->own_slots ? al(sizeof(double) * (size_t)(4 * (P->groups[0].nblocks + P->groups[1].nblocks
                                                              + P->groups[2].nblocks)) * P->nef_max) : 0;
    D.gctr = al(sizeof(double) * P->gctr_size);
    D.cnt = al(sizeof(int) * 4);
    D.ne = al(sizeof(int) * std::max<size_t>(P->outs.size(), 1));
    D.scr = fo ? al(sizeof(double)) : al(sizeof(double) * D.spw * D.out_blocks * 4);
    D.wwarps = 0;
    D.wscr = 0;
    const bool grad = P->mode == CG_MODE_GRAD || P->mode == CG_MODE_GRADA;
    /* per-warp slots: J mode holds (e0|f0) and two transfer buffers, the adjoint a cotangent */
    D.wstride = P->jmode ? (int64_t)P->nef_max + 2 * (int64_t)P->hrr_max : (int64_t)P->max_nf;
    if (P->jmode || (grad && !P->gradj && P->max_nf > CG_W_SMEM)) {
        D.wwarps = g_ctx.sm_count * 4 * (P->groups[0].blocks_per_sm + P->groups[1].blocks_per_sm
                                         + P->groups[2].blocks_per_sm);
        D.wscr = al(sizeof(double) * (size_t)D.wwarps * D.wstride);
    }
    if (P->jmode || grad) D.gctr = al(sizeof(double));   /* no per-task accumulators */
    D.upload = D.pairs + D.prims + D.tasks + D.outs + D.pq + D.gcl + D.gch + D.gen + D.ecl + D.egr + D.epm + D.hpg + D.erd + D.emp;
    D.total = D.upload + D.gctr + D.cnt + D.ne + D.scr + D.wscr + D.done + D.oscr + D.wslot;
    return D;
}

static size_t plan_device_bytes(const CINTGPUPlan *P) { return dev_layout(P).total; }
static size_t plan_upload_bytes(const CINTGPUPlan *P) { return dev_layout(P).upload; }

/* Device pointers of every plan array inside one region laid out by D (upload part first). */
static void carve_plan(CINTGPUPlan *P, const DevLayout &D, char *p)
{
    P->out_blocks = D.out_blocks;
    P->scratch_per_warp = D.spw;
    P->d_pairs = (CGPair *)p; p += D.pairs;
    P->d_prims = (CGPrimPair *)p; p += D.prims;
    P->d_tasks = (CGTask *)p; p += D.tasks;
    P->d_outs = (CGOutTask *)p; p += D.outs;
    P->d_pqlist = (int *)p; p += D.pq;
    P->d_gclass = (CGGradClass *)p; p += D.gcl;
    P->d_gchunk = (CGGradChunk *)p; p += D.gch;
    P->d_gent = (CGGradEnt *)p; p += D.gen;
    P->d_eclass = (CGEriClass *)p; p += D.ecl;
    P->d_egroup = (CGEriGroup *)p; p += D.egr;
    P->d_eperm = (int *)p; p += D.epm;
    P->d_hprog = (int *)p; p += D.hpg;
    P->d_eround = (int *)p; p += D.erd;
    P->d_empty = (int *)p; p += D.emp;
    P->d_gctr = (double *)p; p += D.gctr;
    P->d_counters = (int *)p; p += D.cnt;
    P->d_nonempty = (int *)p; p += D.ne;
    P->d_scratch = (double *)p; p += D.scr;
    P->d_wscratch = (double *)p; p += D.wscr;
    P->d_done = (int *)p; p += D.done;
    P->d_oscr = D.oscr ? (double *)p : nullptr; p += D.oscr;
    P->d_wslot = D.wslot ? (double *)p : nullptr; p += D.wslot;
    P->wscratch_stride = D.wstride;
    P->wscratch_warps = D.wwarps;
}

/* Host image of the upload part of the region (D.upload bytes). */
static void fill_image(const CINTGPUPlan *P, const DevLayout &D, char *q)
{
    memcpy(q, P->pairs.data(), sizeof(CGPair) * P->pairs.size()); q += D.pairs;
    memcpy(q, P->prims.data(), sizeof(CGPrimPair) * P->prims.size()); q += D.prims;
    memcpy(q, P->tasks.data(), sizeof(CGTask) * P->tasks.size()); q += D.tasks;
    memcpy(q, P->outs.data(), sizeof(CGOutTask) * P->outs.size()); q += D.outs;
    memcpy(q, P->pqlist.data(), sizeof(int) * P->pqlist.size()); q += D.pq;
    memcpy(q, P->gclass.data(), sizeof(CGGradClass) * P->gclass.size()); q += D.gcl;
    memcpy(q, P->gchunk.data(), sizeof(CGGradChunk) * P->gchunk.size()); q += D.gch;
    memcpy(q, P->gent.data(), sizeof(CGGradEnt) * P->gent.size()); q += D.gen;
    memcpy(q, P->eclass.data(), sizeof(CGEriClass) * P->eclass.size()); q += D.ecl;
    memcpy(q, P->egroup.data(), sizeof(CGEriGroup) * P->egroup.size()); q += D.egr;
    memcpy(q, P->eperm.data(), sizeof(int) * P->eperm.size()); q += D.epm;
    memcpy(q, P->hprog.data(), sizeof(int) * P->hprog.size()); q += D.hpg;
    memcpy(q, P->eround.data(), sizeof(int) * P->eround.size()); q += D.erd;
    memcpy(q, P->empty_outs.data(), sizeof(int) * P->empty_outs.size());
}

/* Place the plan in device memory (a caller arena or its own allocation) and copy the host
 * images: pinned + async on `stream` for the drop-in, synchronous otherwise. */
static int upload_plan(CINTGPUPlan *P, char *arena, size_t arena_size, cudaStream_t stream,
                       bool async_from_pinned, char *pinned)
{
    DevLayout D = dev_layout(P);
    P->out_blocks = D.out_blocks;
    P->scratch_per_warp = D.spw;
    if (arena) {
        if (D.total > arena_size) { set_error("arena too small"); return CINTGPU_ERR_NOMEM; }
        P->dbuf = arena; P->dbuf_size = arena_size; P->owns_dbuf = false;
    } else {
        cudaError_t e = cudaMalloc(&P->dbuf, D.total);
        if (e != cudaSuccess) {
            set_error("cudaMalloc(%zu) failed: %s", D.total, cudaGetErrorString(e));
            P->dbuf = nullptr;
            return CINTGPU_ERR_NOMEM;
        }
        P->dbuf_size = D.total; P->owns_dbuf = true;
    }
    carve_plan(P, D, P->dbuf);
    std::vector<char> tmp;
    char *src;
    if (async_from_pinned) src = pinned;
    else { tmp.resize(D.upload); src = tmp.data(); }
    fill_image(P, D, src);
    if (async_from_pinned) {
        CUDA_OK(cudaMemcpyAsync(P->dbuf, src, D.upload, cudaMemcpyHostToDevice, stream));
    } else {
        CUDA_OK(cudaMemcpy(P->dbuf, src, D.upload, cudaMemcpyHostToDevice));
    }
    return 0;
}

static int launch_grad_group(CINTGPUPlan *P, int g, cudaStream_t stream)
{
    const TaskGroup &G = P->groups[g];
    if (G.ntasks == 0) return 0;
    CGGradLaunch L;
    L.tasks = P->d_tasks + G.task0;
    L.ntasks = G.ntasks;
    L.pairs = P->d_pairs;
    L.prims = P->d_prims;
    L.pqlist = P->d_pqlist;
    L.counter = P->d_counters + g;
    L.status = P->d_counters + 2;
    L.rys_coef = g_ctx.rys_coef;
    L.common_base = M_PI * M_PI * M_PI * 2 / 1.7724538509055160272981674833411451;
    L.omega2 = P->omega2;
    L.expcut = P->expcutoff;
    L.ws_doubles = G.ws;
    L.dm = P->cur_dm;
    L.nao = P->nao_cart;
    L.grad = P->cur_grad;
    L.galpha = P->cur_galpha;
    L.gclass = P->d_gclass;
    L.gchunk = P->d_gchunk;
    L.gent = P->d_gent;
    L.wglobal = P->d_wscratch;
    if (g == 1 && P->d_wscratch)
        L.wglobal += (size_t)g_ctx.sm_count * 4 * P->groups[0].blocks_per_sm * P->max_nf;
    L.wstride = P->max_nf;
    const int nblocks = G.nblocks;
    int rc = cg_launch_grad(&L, grad_kernel_mode(P), nblocks, stream);
    if (rc) { set_error("adjoint kernel launch failed: %s", cudaGetErrorString((cudaError_t)rc)); return CINTGPU_ERR_CUDA; }
    return 0;
}

static int launch_group(CINTGPUPlan *P, int g, cudaStream_t stream)
{
    if (P->mode == CG_MODE_GRAD || P->mode == CG_MODE_GRADA) return launch_grad_group(P, g, stream);
    const TaskGroup &G = P->groups[g];
    if (G.ntasks == 0) return 0;
    CGLaunch L;
    memset(&L, 0, sizeof(L));
    L.tasks = P->d_tasks;
    L.task0 = G.task0;
    L.ntasks = G.ntasks;
    L.pairs = P->d_pairs;
    L.prims = P->d_prims;
    L.pqlist = P->d_pqlist;
    L.gctr = P->d_gctr;
    L.counter = P->d_counters + (g == 2 ? 3 : g);   /* [2] is the status word */
    L.nonempty = P->d_nonempty;
    L.status = P->d_counters + 2;
    L.rys_coef = g_ctx.rys_coef;
    L.common_base = M_PI * M_PI * M_PI * 2 / 1.7724538509055160272981674833411451;
    L.omega2 = P->omega2;
    L.expcut = P->expcutoff;
    L.three = P->three;
    L.two = P->two;
    L.ws_doubles = G.ws;
    L.jmode = P->jmode;
    L.wscratch = P->d_wscratch;
    if (P->jmode && g >= 1)   /* the groups may run concurrently: separate warp slots */
        L.wscratch += (size_t)g_ctx.sm_count * 4
                      * (P->groups[0].blocks_per_sm + (g == 2 ? P->groups[1].blocks_per_sm : 0)) * P->wscratch_stride;
    L.wscratch_stride = P->wscratch_stride;
    L.dm = P->cur_dm;
    L.vj = P->cur_vj;
    L.vk = P->cur_vk;
    L.nao = P->nao_cart;
    L.eclass = P->d_eclass;
    L.egroup = P->d_egroup;
    L.eperm = P->d_eperm;
    L.hprog = P->d_hprog;
    L.eround = P->d_eround;
    L.fuse_out = fused(P) ? 1 : 0;
    L.outs = P->d_outs;
    L.done = P->d_done;
    L.oscr = P->d_oscr;
    if (L.oscr && g >= 1)
        L.oscr += (size_t)4 * (P->groups[0].nblocks + (g == 2 ? P->groups[1].nblocks : 0)) * P->scratch_per_warp;
    L.oscr_stride = P->scratch_per_warp;
    /* own slots: per warp of this launch, after those of the groups launched beside it */
    L.wslot = P->d_wslot;
    L.wslot_stride = P->nef_max;
    if (L.wslot && g >= 1)
        L.wslot += (size_t)4 * (P->groups[0].nblocks + (g == 2 ? P->groups[1].nblocks : 0)) * P->nef_max;
    L.nf_max = P->max_nf;
    L.out = P->cur_out;
    L.ncomp = P->ncomp;
    L.comp_stride = P->out_size;
    L.hrr_off1 = P->nef_max;
    L.hrr_off2 = (int64_t)P->nef_max + P->hrr_max;
    const int nblocks = G.nblocks;
    int rc = cg_launch_eri(&L, g == 2 ? CG_MODE_ERIP : P->mode, nblocks, stream);
    if (rc) { set_error("ERI kernel launch failed: %s", cudaGetErrorString((cudaError_t)rc)); return CINTGPU_ERR_CUDA; }
    return 0;
}

/* memsets, the two task groups (concurrently when the plan owns a side stream), the output
 * kernel.  Everything is enqueued on `stream`; nothing synchronises with the host. */
static int execute_plan(CINTGPUPlan *P, double *out_dev, cudaStream_t stream)
{
    CUDA_OK(cudaMemsetAsync(P->d_nonempty, 0, sizeof(int) * std::max<size_t>(P->outs.size(), 1), stream));
    CUDA_OK(cudaMemsetAsync(P->d_counters, 0, sizeof(int) * 4, stream));
    const bool fo = fused(P);
    if (fo) CUDA_OK(cudaMemsetAsync(P->d_done, 0, sizeof(int) * std::max<size_t>(P->outs.size(), 1), stream));
    P->cur_out = out_dev;
    /* the 48 KB and per-primitive groups run on the side stream beside the regular group: their
     * CTAs take SMs as the regular group's drain, so the launches' tails overlap */
    const bool side_work = P->groups[1].ntasks > 0 || P->groups[2].ntasks > 0;
    bool fork = P->side && side_work && P->groups[0].ntasks > 0;
    if (P->ev_t0) CUDA_OK(cudaEventRecord(P->ev_t0, stream));
    if (fork) {
        CUDA_OK(cudaEventRecord(P->ev_fork, stream));
        CUDA_OK(cudaStreamWaitEvent(P->side, P->ev_fork, 0));
        int rc = launch_group(P, 1, P->side);
        if (!rc) rc = launch_group(P, 2, P->side);
        if (rc) return rc;
        CUDA_OK(cudaEventRecord(P->ev_join, P->side));
        rc = launch_group(P, 0, stream);
        if (rc) return rc;
        CUDA_OK(cudaStreamWaitEvent(stream, P->ev_join, 0));
    } else {
        int rc = launch_group(P, 1, stream);
        if (!rc) rc = launch_group(P, 0, stream);
        if (!rc) rc = launch_group(P, 2, stream);
        if (rc) return rc;
    }
    if (P->ev_t1) {
        CUDA_OK(cudaEventRecord(P->ev_t1, stream));
        P->timed = true;
    }
    if (P->jmode || P->mode == CG_MODE_GRAD || P->mode == CG_MODE_GRADA) return 0;
    if (fo && P->empty_outs.empty()) return 0;
    int rc = cg_launch_output(P->d_outs, fo ? P->d_empty : nullptr,
                              fo ? (int)P->empty_outs.size() : (int)P->outs.size(), P->d_gctr, P->d_nonempty, P->d_scratch,
                              P->scratch_per_warp, P->max_nf, P->d_eclass, P->d_eperm, P->d_hprog, P->out_blocks,
                              out_dev, P->ncomp, P->out_size, stream);
    if (rc) { set_error("output kernel launch failed: %s", cudaGetErrorString((cudaError_t)rc)); return CINTGPU_ERR_CUDA; }
    return 0;
}

/* ------------------------------------------------------------------ per-thread drop-in state */
namespace {
struct ThreadCtx {
    cudaStream_t stream = nullptr;
    char *arena = nullptr;
    size_t arena_size = 0;
    double *dout = nullptr;
    size_t dout_size = 0;
    char *pinned = nullptr;
    size_t pinned_size = 0;
    double *hout = nullptr;
    size_t hout_size = 0;
    ~ThreadCtx()
    {
        /* process teardown may already have destroyed the context; ignore errors */
        if (arena) cudaFree(arena);
        if (dout) cudaFree(dout);
        if (pinned) cudaFreeHost(pinned);
        if (hout) cudaFreeHost(hout);
        if (stream) cudaStreamDestroy(stream);
    }
};
thread_local ThreadCtx tl_ctx;

int grow_dev(char **p, size_t *cap, size_t need)
{
    if (need <= *cap) return 0;
    if (*p) cudaFree(*p);
    size_t n = std::max(need, *cap * 2);
    if (cudaMalloc(p, n) != cudaSuccess) { *p = nullptr; *cap = 0; set_error("cudaMalloc(%zu) failed", n); return CINTGPU_ERR_NOMEM; }
    *cap = n;
    return 0;
}
int grow_host(char **p, size_t *cap, size_t need)
{
    if (need <= *cap) return 0;
    if (*p) cudaFreeHost(*p);
    size_t n = std::max(need, *cap * 2);
    if (cudaMallocHost(p, n) != cudaSuccess) { *p = nullptr; *cap = 0; set_error("cudaMallocHost(%zu) failed", n); return CINTGPU_ERR_NOMEM; }
    *cap = n;
    return 0;
}

/* libcint cache-size formula of CINT2e_drv / CINT3c2e_drv / CINT2c2e_drv (src/cint2e.c:779-816,
 * src/cint3c2e.c:545-567, src/cint2c2e.c:244-246 with int1e_cache_size, src/cint1e.c:163-183) so
 * out == NULL queries return the same number. */
CACHE_SIZE_T cache_size_query(int kind, const int *shls, const int *bas)
{
    if (kind_shells(kind) == 2) {
        /* CINTinit_int2c2e_EnvVars: g_size = nroots (li+1) (lk+1), i and k in the 1e slots */
        const int *bi = bas + BAS_SLOTS * shls[0], *bk = bas + BAS_SLOTS * shls[1];
        const int64_t li = bi[ANG_OF], lk = bk[ANG_OF];
        const int64_t ip = bi[NPRIM_OF], kp = bk[NPRIM_OF], ic = bi[NCTR_OF], kc = bk[NCTR_OF];
        const int64_t nf = (int64_t)ncart_l((int)li) * ncart_l((int)lk);
        const int64_t nc = nf * ic * kc;
        const int64_t leng = ((li + lk) / 2 + 1) * (li + 1) * (lk + 1) * 3 * 2;
        const int64_t pdata = ip * kp * 5 + ip * ic + kp * kc + (ip + kp) * 2 + nf * 3;
        return (CACHE_SIZE_T)std::max(nc + leng + nf * nc + nf * ic + nf + pdata, nc + nf * 8 * 2);
    }
    int three = kind_shells(kind) == 3;
    /* ng increments of libcint's autocode (grad2.c, int3c2e.c): IINC for the ip1 kinds, KINC
     * for ip2; one g-array shift and 3 components for both */
    int iinc = kind == CINTGPU_INT2E_IP1_SPH || kind == CINTGPU_INT2E_IP1_CART
            || kind == CINTGPU_INT3C2E_IP1_SPH || kind == CINTGPU_INT3C2E_IP1_CART;
    const int ipip = kind == CINTGPU_INT2E_IPIP1_SPH || kind == CINTGPU_INT2E_IPIP1_CART;
    if (ipip) iinc = 2;   /* hess.c ng = {2, 0, 0, 0, 2 (GSHIFT), 1, 1, 9} */
    int kinc = kind == CINTGPU_INT2E_IP2_SPH || kind == CINTGPU_INT2E_IP2_CART
            || kind == CINTGPU_INT3C2E_IP2_SPH || kind == CINTGPU_INT3C2E_IP2_CART;
    int ip1 = iinc || kinc;
    int nsh = three ? 3 : 4;
    int l[4] = {0, 0, 0, 0}, np[4] = {1, 1, 1, 1}, nc[4] = {1, 1, 1, 1};
    for (int a = 0; a < nsh; a++) {
        const int *b = bas + BAS_SLOTS * shls[a];
        l[a] = b[ANG_OF]; np[a] = b[NPRIM_OF]; nc[a] = b[NCTR_OF];
    }
    int ncomp = ipip ? 9 : (ip1 ? 3 : 1), gbits = ipip ? 2 : (ip1 ? 1 : 0);
    int lic = l[0] + iinc, ljc = l[1], lkc = l[2] + kinc, llc = l[3];
    size_t nf = (size_t)ncart_l(l[0]) * ncart_l(l[1]) * ncart_l(l[2]) * (three ? 1 : ncart_l(l[3]));
    size_t ncx = nf * nc[0] * nc[1] * nc[2] * (three ? 1 : nc[3]);
    size_t gsize;
    int nroots;
    if (three) {
        /* CINTinit_int3c2e_EnvVars (src/g3c2e.c:21-132): lk_ceil = 0, ll_ceil = k_l + KINC */
        nroots = (lic + ljc + lkc) / 2 + 1;
        int dli, dlj;
        if (lic > ljc) { dli = lic + ljc + 1; dlj = ljc + 1; } else { dli = lic + 1; dlj = lic + ljc + 1; }
        gsize = (size_t)nroots * dli * (lkc + 1) * dlj;
        size_t leng = gsize * 3 * ((1 << gbits) + 1);
        size_t len0 = nf * ncomp;
        size_t ps = (size_t)np[0] * np[1] * 5 + np[0] * nc[0] + np[1] * nc[1] + np[2] * nc[2]
                  + (np[0] + np[1]) * 2 + np[2] + nf * 3 + 16;
        return (CACHE_SIZE_T)std::max(leng + len0 + ncx * ncomp * 3 + ps, ncx * ncomp + nf * 3);
    }
    nroots = (lic + ljc + lkc + llc) / 2 + 1;
    int dli, dlj, dlk, dll;
    if (lkc > llc) { dlk = lkc + llc + 1; dll = llc + 1; } else { dlk = lkc + 1; dll = lkc + llc + 1; }
    if (lic > ljc) { dli = lic + ljc + 1; dlj = ljc + 1; } else { dli = lic + 1; dlj = lic + ljc + 1; }
    gsize = (size_t)nroots * dli * dlk * dll * dlj;
    size_t leng = gsize * 3 * ((1 << gbits) + 1);
    size_t len0 = nf * ncomp;
    size_t ps = ((size_t)np[0] * np[1] + (size_t)np[2] * np[3]) * 5 + np[0] * nc[0] + np[1] * nc[1]
              + np[2] * nc[2] + np[3] * nc[3] + (np[0] + np[1] + np[2] + np[3]) * 2 + nf * 3;
    return (CACHE_SIZE_T)std::max(leng + len0 + ncx * ncomp * 3 + ps, ncx * ncomp + nf * 4);
}

/* drop-in calls that failed since the library was loaded */
std::atomic<int64_t> g_dropin_failures{0};

/* One shell block through the GPU (the plain drop-in path). */
CACHE_SIZE_T dropin(int kind, double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm,
                    FINT *bas, FINT nbas, double *env, CINTOpt *opt = nullptr)
{
    if (out == NULL) return cache_size_query(kind, shls, bas);
    const int nsh = kind_shells(kind);
    int ncomp = (kind == CINTGPU_INT2E_IP1_SPH || kind == CINTGPU_INT2E_IP1_CART
                 || (kind >= CINTGPU_INT2E_IP2_SPH && kind <= CINTGPU_INT3C2E_IP2_CART)) ? 3 : 1;
    if (kind == CINTGPU_INT2E_IPIP1_SPH || kind == CINTGPU_INT2E_IPIP1_CART) ncomp = 9;
    int sph = kind_sph(kind);
    int counts[4] = {1, 1, 1, 1};
    for (int a = 0; a < nsh; a++) {
        const int *b = bas + BAS_SLOTS * shls[a];
        int l = b[ANG_OF];
        counts[a] = (sph ? nsph_l(l) : ncart_l(l)) * b[NCTR_OF];
    }
    /* the caller's dims hold one entry per shell (2, 3 or 4); padded with 1 */
    int d[4] = {1, 1, 1, 1};
    for (int a = 0; a < nsh; a++) d[a] = dims ? dims[a] : counts[a];
    int64_t nout = (int64_t)d[0] * d[1] * d[2] * d[3];
    auto fill = [&](double v) {
        for (int comp = 0; comp < ncomp; comp++)
            for (int l = 0; l < counts[3]; l++)
                for (int k = 0; k < counts[2]; k++)
                    for (int j = 0; j < counts[1]; j++)
                        for (int i = 0; i < counts[0]; i++)
                            out[comp * nout + i + (int64_t)d[0] * (j + (int64_t)d[1] * (k + (int64_t)d[2] * l))] = v;
    };
    auto zero_fill = [&]() { fill(0.0); };
    /* A failed call (no device, a CUDA error, bad input) must not look like a screened block,
     * which libcint returns as zeros with 0: the block is filled with NaN, the call returns 0,
     * the failure is counted (cintgpu_dropin_failures) and the first one is reported on stderr. */
    auto failed = [&]() -> CACHE_SIZE_T {
        fill(std::numeric_limits<double>::quiet_NaN());
        if (g_dropin_failures.fetch_add(1) == 0)
            fprintf(stderr, "libcintgpu: a drop-in integral call failed (%s); its block is filled "
                            "with NaN (cintgpu_dropin_failures counts such calls)\n", tl_error.c_str());
        return 0;
    };
    if (ensure_init()) return failed();
    ThreadCtx &T = tl_ctx;
    if (!T.stream && cudaStreamCreateWithFlags(&T.stream, cudaStreamNonBlocking) != cudaSuccess) {
        set_error("cudaStreamCreate failed");
        return failed();
    }
    CINTGPUPlan P;
    P.fuse_out = false;   /* one quartet: a separate transform needs far less scratch */
    std::shared_ptr<OptState> os = opt_state(opt);
    int rc = build_plan(&P, kind, shls, 1, NULL, atm, natm, bas, nbas, env,
                        (int64_t)g_ctx.sm_count * 8, os.get());
    if (rc) return failed();
    /* libcint's return value: 0 when no primitive quartet survives the screening, which the
     * planner decides on the host (a quartet without tasks); such a block is zero-filled here
     * without a GPU round trip, and a block with tasks is non-empty */
    if (P.empty_outs.size() == P.outs.size()) { zero_fill(); return 0; }
    size_t need = plan_device_bytes(&P);
    size_t up = plan_upload_bytes(&P);
    size_t outb = sizeof(double) * P.out_size * ncomp;
    if (grow_dev(&T.arena, &T.arena_size, need) || grow_dev((char **)&T.dout, &T.dout_size, outb)
        || grow_host(&T.pinned, &T.pinned_size, up)
        || grow_host((char **)&T.hout, &T.hout_size, outb))
        return failed();
    rc = upload_plan(&P, T.arena, T.arena_size, T.stream, true, T.pinned);
    if (!rc) rc = execute_plan(&P, T.dout, T.stream);
    if (!rc && cudaMemcpyAsync(T.hout, T.dout, outb, cudaMemcpyDeviceToHost, T.stream) != cudaSuccess) rc = -1;
    if (!rc && cudaStreamSynchronize(T.stream) != cudaSuccess) { set_error("kernel execution failed: %s", cudaGetErrorString(cudaGetLastError())); rc = -1; }
    P.dbuf = nullptr;
    if (rc) return failed();
    /* dense GPU block -> caller layout with dims */
    for (int comp = 0; comp < ncomp; comp++) {
        const double *src = T.hout + comp * P.out_size;
        for (int l = 0; l < counts[3]; l++)
            for (int k = 0; k < counts[2]; k++)
                for (int j = 0; j < counts[1]; j++) {
                    const double *s = src + counts[0] * (j + (int64_t)counts[1] * (k + (int64_t)counts[2] * l));
                    double *o = out + comp * nout + (int64_t)d[0] * (j + (int64_t)d[1] * (k + (int64_t)d[2] * l));
                    memcpy(o, s, sizeof(double) * counts[0]);
                }
    }
    return 1;
}

void make_opt(CINTOpt **opt, FINT nbas)
{
    CINTOpt *o = (CINTOpt *)calloc(1, sizeof(CINTOpt));
    o->nbas = nbas;
    std::lock_guard<std::mutex> lk(g_opt_mu);
    g_opt_states[o] = std::make_shared<OptState>();
    *opt = o;
}
}  // namespace

/* ================================================================== C ABI */
extern "C" {

const char *cintgpu_last_error(void) { return tl_error.c_str(); }

int64_t cintgpu_dropin_failures(void) { return g_dropin_failures.load(); }

int cintgpu_device_sm_count(void)
{
    if (ensure_init()) return 0;
    return g_ctx.sm_count;
}

int cintgpu_rys_nmax(void) { return cg_rys_nmax(); }

int cintgpu_rys_roots_dev(int nroots, const double *xs_dev, int count, double *s_dev,
                          double *w_dev, void *stream)
{
    int rc = ensure_init();
    if (rc) return rc;
    if (nroots < 1 || nroots > cg_rys_nmax()) { set_error("nroots %d outside 1..%d", nroots, cg_rys_nmax()); return CINTGPU_ERR_ARG; }
    rc = cg_launch_roots(xs_dev, count, nroots, g_ctx.rys_coef, s_dev, w_dev, (cudaStream_t)stream);
    if (rc) { set_error("roots kernel failed"); return CINTGPU_ERR_CUDA; }
    return 0;
}

static int plan_create(CINTGPUPlan **plan, int kind, const int *shls, int64_t n,
                       const int64_t *offsets, const int *atm, int natm, const int *bas,
                       int nbas, const double *env, int ws_kb, int separate_output,
                       const int *wide = nullptr, int nwide = 0)
{
    *plan = nullptr;
    int rc = ensure_init();
    if (rc) return rc;
    CINTGPUPlan *P = new CINTGPUPlan();
    P->ws_kb = ws_kb;
    if (wide && nwide > 0) P->wide.assign(wide, wide + nwide);
    P->plan_threads = (int)std::thread::hardware_concurrency();
    /* CINTGPU_SEPARATE_OUTPUT=1: transform outputs in their own kernel (tuning) */
    if (const char *e = getenv("CINTGPU_SEPARATE_OUTPUT")) P->fuse_out = atoi(e) == 0;
    if (separate_output) P->fuse_out = false;
    int64_t target = n < (int64_t)g_ctx.sm_count * 16 ? (int64_t)g_ctx.sm_count * 8 : 0;
    rc = build_plan(P, kind, shls, n, offsets, atm, natm, bas, nbas, env, target);
    if (!rc) rc = upload_plan(P, nullptr, 0, 0, false, nullptr);
    if (!rc && (cudaStreamCreateWithFlags(&P->side, cudaStreamNonBlocking) != cudaSuccess
                || cudaEventCreateWithFlags(&P->ev_fork, cudaEventDisableTiming) != cudaSuccess
                || cudaEventCreateWithFlags(&P->ev_join, cudaEventDisableTiming) != cudaSuccess
                || cudaEventCreate(&P->ev_t0) != cudaSuccess || cudaEventCreate(&P->ev_t1) != cudaSuccess)) {
        set_error("stream/event creation failed");
        rc = CINTGPU_ERR_CUDA;
    }
    if (rc) { free_plan_device(P); delete P; return rc; }
    *plan = P;
    return 0;
}

int cintgpu_plan_create(CINTGPUPlan **plan, int kind, const int *shls, int64_t n,
                        const int64_t *offsets, const int *atm, int natm, const int *bas,
                        int nbas, const double *env)
{
    return plan_create(plan, kind, shls, n, offsets, atm, natm, bas, nbas, env, 0, 0);
}

int cintgpu_plan_create_tuned(CINTGPUPlan **plan, int kind, const int *shls, int64_t n,
                              const int64_t *offsets, const int *atm, int natm, const int *bas,
                              int nbas, const double *env, int ws_kb, int separate_output)
{
    if (plan) *plan = nullptr;
    if (ws_kb != 0 && (ws_kb < 8 || ws_kb > 48)) {
        set_error("ws_kb %d outside 8..48 (0 = default)", ws_kb);
        return CINTGPU_ERR_ARG;
    }
    if (separate_output != 0 && separate_output != 1) {
        set_error("separate_output must be 0 or 1");
        return CINTGPU_ERR_ARG;
    }
    return plan_create(plan, kind, shls, n, offsets, atm, natm, bas, nbas, env, ws_kb,
                       separate_output);
}

int cintgpu_plan_create_classes(CINTGPUPlan **plan, int kind, const int *shls, int64_t n,
                                const int64_t *offsets, const int *atm, int natm, const int *bas,
                                int nbas, const double *env, int ws_kb, int separate_output,
                                const int *wide, int nwide)
{
    if (plan) *plan = nullptr;
    if (ws_kb != 0 && (ws_kb < 8 || ws_kb > 48)) {
        set_error("ws_kb %d outside 8..48 (0 = default)", ws_kb);
        return CINTGPU_ERR_ARG;
    }
    if (separate_output != 0 && separate_output != 1) {
        set_error("separate_output must be 0 or 1");
        return CINTGPU_ERR_ARG;
    }
    if (nwide < 0 || (nwide > 0 && !wide)) {
        set_error("wide: %d class keys without an array", nwide);
        return CINTGPU_ERR_ARG;
    }
    for (int i = 0; i < nwide; i++)
        if (wide[i] < 0 || wide[i] >= 8 * 8 * 8 * 8) {
            set_error("class key %d outside 0..4095", wide[i]);
            return CINTGPU_ERR_ARG;
        }
    return plan_create(plan, kind, shls, n, offsets, atm, natm, bas, nbas, env, ws_kb,
                       separate_output, wide, nwide);
}

int64_t cintgpu_plan_output_size(const CINTGPUPlan *plan) { return plan->out_size; }
int cintgpu_plan_ncomp(const CINTGPUPlan *plan) { return plan->ncomp; }
double cintgpu_plan_flops(const CINTGPUPlan *plan) { return plan->flops; }
double cintgpu_plan_flops_libcint(const CINTGPUPlan *plan) { return plan->flops_ref; }
int64_t cintgpu_plan_prim_quartets(const CINTGPUPlan *plan) { return plan->prim_quartets; }
int cintgpu_plan_launches(const CINTGPUPlan *plan)
{
    /* the task groups with work, and the output kernel when execute_plan launches it */
    const bool contracting = plan->jmode || plan->mode == CG_MODE_GRAD || plan->mode == CG_MODE_GRADA;
    const bool output = !contracting && !(fused(plan) && plan->empty_outs.empty());
    return (plan->groups[0].ntasks > 0) + (plan->groups[1].ntasks > 0) + (plan->groups[2].ntasks > 0)
         + (output ? 1 : 0);
}
int64_t cintgpu_plan_upload_bytes(const CINTGPUPlan *plan) { return (int64_t)plan_upload_bytes(plan); }

int cintgpu_plan_execute(CINTGPUPlan *plan, double *out_dev, void *stream)
{
    return execute_plan(plan, out_dev, (cudaStream_t)stream);
}

int cintgpu_plan_nao_cart(const CINTGPUPlan *plan) { return plan->nao_cart; }

float cintgpu_plan_compute_ms(const CINTGPUPlan *plan)
{
    if (!plan || !plan->timed) return -1.0f;
    float ms = -1.0f;
    if (cudaEventSynchronize(plan->ev_t1) != cudaSuccess
        || cudaEventElapsedTime(&ms, plan->ev_t0, plan->ev_t1) != cudaSuccess) {
        set_error("compute timing unavailable: %s", cudaGetErrorString(cudaGetLastError()));
        return -1.0f;
    }
    return ms;
}

int cintgpu_plan_status(const CINTGPUPlan *plan)
{
    int st = 0;
    CUDA_OK(cudaDeviceSynchronize());
    CUDA_OK(cudaMemcpy(&st, plan->d_counters + 2, sizeof(int), cudaMemcpyDeviceToHost));
    return st;
}

/* Diagnostics (not in the public header): info[0..11] = tasks, tasks of groups 0 and 1, adjoint
 * classes / chunks / entries, shared-memory doubles per warp of group 0, CTAs per SM of groups 0
 * and 1, mode, tasks of group 2 (per-primitive int2e), fused outputs (0/1). */
int cintgpu_plan_debug(const CINTGPUPlan *plan, int64_t *info)
{
    info[0] = (int64_t)plan->tasks.size();
    info[1] = plan->groups[0].ntasks;
    info[2] = plan->groups[1].ntasks;
    info[3] = (int64_t)plan->gclass.size();
    info[4] = (int64_t)plan->gchunk.size();
    info[5] = (int64_t)plan->gent.size();
    info[6] = plan->groups[0].ws;
    info[7] = plan->groups[0].blocks_per_sm;
    info[8] = plan->groups[1].blocks_per_sm;
    info[9] = plan->mode;
    info[10] = plan->groups[2].ntasks;
    info[11] = fused(plan) ? 1 : 0;
    return 0;
}

int cintgpu_plan_execute_j(CINTGPUPlan *plan, const double *dm_dev, double *vj_dev, void *stream)
{
    if (plan->jmode != 1) { set_error("plan is not a J_BUILD plan"); return CINTGPU_ERR_ARG; }
    return cintgpu_plan_execute_jk(plan, dm_dev, vj_dev, nullptr, stream);
}

int cintgpu_plan_execute_jk(CINTGPUPlan *plan, const double *dm_dev, double *vj_dev, double *vk_dev,
                            void *stream)
{
    if (!plan->jmode) { set_error("plan is not a J_BUILD, K_BUILD or JK_BUILD plan"); return CINTGPU_ERR_ARG; }
    if (!dm_dev || ((plan->jmode & 1) && !vj_dev) || ((plan->jmode & 2) && !vk_dev)) {
        set_error("the plan needs dm%s%s", (plan->jmode & 1) ? ", vj" : "", (plan->jmode & 2) ? ", vk" : "");
        return CINTGPU_ERR_ARG;
    }
    plan->cur_dm = dm_dev;
    plan->cur_vj = (plan->jmode & 1) ? vj_dev : nullptr;
    plan->cur_vk = (plan->jmode & 2) ? vk_dev : nullptr;
    return execute_plan(plan, nullptr, (cudaStream_t)stream);
}

int cintgpu_plan_execute_grad(CINTGPUPlan *plan, const double *dm_dev, double *grad_dev,
                              double *galpha_dev, void *stream)
{
    if (plan->mode != CG_MODE_GRAD && plan->mode != CG_MODE_GRADA) {
        set_error("plan is not an adjoint plan");
        return CINTGPU_ERR_ARG;
    }
    if (plan->mode == CG_MODE_GRADA && !galpha_dev) { set_error("J_GRAD_EXP needs galpha"); return CINTGPU_ERR_ARG; }
    plan->cur_dm = dm_dev;
    plan->cur_grad = grad_dev;
    plan->cur_galpha = galpha_dev;
    return execute_plan(plan, nullptr, (cudaStream_t)stream);
}

int cintgpu_cart2sph(int l, double *c)
{
    int nc = ncart_l(l);
    if (l < 0 || l > CG_MAX_SHELL_L) return 0;
    if (l <= 1) {
        for (int i = 0; i < nc * nc; i++) c[i] = 0;
        for (int i = 0; i < nc; i++) c[i * nc + i] = 1;
        return nc;
    }
    std::vector<int> nnz, idx;
    std::vector<double> val;
    c2s_rows(nnz, idx, val);
    for (int i = 0; i < (2 * l + 1) * nc; i++) c[i] = 0;
    for (int m = 0; m < 2 * l + 1; m++) {
        int row = l * l + m;
        for (int z = 0; z < nnz[row]; z++) c[m * nc + idx[row * CG_C2S_MAXNNZ + z]] = val[row * CG_C2S_MAXNNZ + z];
    }
    return 2 * l + 1;
}

int cintgpu_plan_nonempty(const CINTGPUPlan *plan, int *flags_host)
{
    std::vector<int> ne(plan->outs.size());
    CUDA_OK(cudaMemcpy(ne.data(), plan->d_nonempty, sizeof(int) * ne.size(), cudaMemcpyDeviceToHost));
    for (int64_t q = 0; q < plan->nitems; q++) flags_host[q] = 0;
    for (size_t o = 0; o < ne.size(); o++) flags_host[plan->out_item[o]] |= ne[o];
    return 0;
}

void cintgpu_plan_destroy(CINTGPUPlan *plan)
{
    if (!plan) return;
    free_plan_device(plan);
    delete plan;
}

namespace {
/* Per-thread buffers of the pipelined host-buffer call: a ring of CG_BATCH_SLOTS slots (device
 * arena + output, pinned image + output), grown on demand and kept between calls. */
#define CG_BATCH_SLOTS 4
struct BatchCtx {
    cudaStream_t s_exec[CG_BATCH_SLOTS] = {}, s_copy = nullptr;   /* one per ring slot */
    cudaEvent_t ev_h2d[CG_BATCH_SLOTS] = {}, ev_exec[CG_BATCH_SLOTS] = {}, ev_d2h[CG_BATCH_SLOTS] = {};
    char *arena[CG_BATCH_SLOTS] = {}, *dout[CG_BATCH_SLOTS] = {};
    char *pin_in[CG_BATCH_SLOTS] = {}, *pin_out[CG_BATCH_SLOTS] = {};
    size_t arena_cap[CG_BATCH_SLOTS] = {}, dout_cap[CG_BATCH_SLOTS] = {};
    size_t pin_in_cap[CG_BATCH_SLOTS] = {}, pin_out_cap[CG_BATCH_SLOTS] = {};
    ~BatchCtx()
    {
        /* process teardown may already have destroyed the context; ignore errors */
        for (int s = 0; s < CG_BATCH_SLOTS; s++) {
            if (arena[s]) cudaFree(arena[s]);
            if (dout[s]) cudaFree(dout[s]);
            if (pin_in[s]) cudaFreeHost(pin_in[s]);
            if (pin_out[s]) cudaFreeHost(pin_out[s]);
            if (ev_h2d[s]) cudaEventDestroy(ev_h2d[s]);
            if (ev_exec[s]) cudaEventDestroy(ev_exec[s]);
            if (ev_d2h[s]) cudaEventDestroy(ev_d2h[s]);
        }
        for (int s = 0; s < CG_BATCH_SLOTS; s++)
            if (s_exec[s]) cudaStreamDestroy(s_exec[s]);
        if (s_copy) cudaStreamDestroy(s_copy);
    }
    int init()
    {
        if (s_copy && ev_d2h[CG_BATCH_SLOTS - 1]) return 0;   /* set up by an earlier call */
        bool ok = s_copy || cudaStreamCreateWithFlags(&s_copy, cudaStreamNonBlocking) == cudaSuccess;
        for (int s = 0; s < CG_BATCH_SLOTS && ok; s++)
            ok = s_exec[s] || cudaStreamCreateWithFlags(&s_exec[s], cudaStreamNonBlocking) == cudaSuccess;
        if (!ok) {
            set_error("stream creation failed");
            return CINTGPU_ERR_CUDA;
        }
        for (int s = 0; s < CG_BATCH_SLOTS; s++)
            if ((!ev_h2d[s] && cudaEventCreateWithFlags(&ev_h2d[s], cudaEventDisableTiming) != cudaSuccess)
                || (!ev_exec[s] && cudaEventCreateWithFlags(&ev_exec[s], cudaEventDisableTiming) != cudaSuccess)
                || (!ev_d2h[s] && cudaEventCreateWithFlags(&ev_d2h[s], cudaEventDisableTiming) != cudaSuccess)) {
                set_error("event creation failed");
                return CINTGPU_ERR_CUDA;
            }
        return 0;
    }
};
thread_local BatchCtx tl_batch;

/* doubles of one component of item q's output block (libcint's dims for the kind) */
int64_t item_block(int kind, const int *q, const int *bas)
{
    const bool sph = kind_sph(kind);
    int64_t b = 1;
    for (int a = 0; a < kind_shells(kind); a++) {
        const int *s = bas + BAS_SLOTS * q[a];
        b *= (int64_t)(sph ? nsph_l(s[ANG_OF]) : ncart_l(s[ANG_OF])) * s[NCTR_OF];
    }
    return b;
}
}  // namespace

/* Host-buffer form over a packed output.  The item list is cut into chunks (512 items, growing
 * by a quarter per chunk up to 12288); chunk c uses slot c % CG_BATCH_SLOTS of a ring and that
 * slot's execution stream (four streams overlap more of the chunks' launch tails than two).
 *   builder threads  build chunk plans and, once the slot's previous upload has completed, write
 *                    the plan's image into the slot's pinned buffer;
 *   the caller       uploads each image, executes the plan and queues the copy back, never
 *                    waiting on the GPU except for a slot whose previous chunk is not scattered;
 *   scatter threads  wait for each chunk's copy and move it into out_host.
 * So planning, image writing and scattering all overlap the GPU, and one chunk's kernel tail
 * overlaps the next chunk on the other stream. */
static int batch_host_pipelined(int kind, double *out_host, const int *shls, int64_t n,
                                const int *atm, int natm, const int *bas, int nbas,
                                const double *env, double *out_dev = nullptr)
{
    /* out_dev: the blocks go straight into this device buffer (one component), no copy back */
    BatchCtx &X = tl_batch;
    int rc = X.init();
    if (rc) return rc;
    const int nsh = kind_shells(kind);
    for (int64_t q = 0; q < n; q++)
        for (int a = 0; a < nsh; a++)
            if (shls[nsh * q + a] < 0 || shls[nsh * q + a] >= nbas) {
                set_error("item %lld: shell %d outside 0..%d", (long long)q, shls[nsh * q + a], nbas - 1);
                return CINTGPU_ERR_ARG;
            }
    struct Chunk {
        int64_t i0 = 0, n = 0, base = 0, out_size = 0;
        int ncomp = 1;
        double t_ready = 0, t_enq = 0;     /* ms since the call started (trace) */
        CINTGPUPlan *P = nullptr;
        DevLayout D;
        int rc = 0;
        std::string err;
        bool image = false, h2d = false, d2h = false, scattered = false;
    };
    /* chunk sizes 512, 640, 800, ... (x 1.25) up to 12288 items: the GPU starts after one small
     * plan, and each later chunk's plan (built by one thread) is ready before the GPU needs it */
    std::vector<Chunk> ch;
    int64_t total = 0;
    /* two- and three-centre items are one to two orders of magnitude cheaper than quartets:
     * their chunks may grow 20x larger before one chunk's plan outlasts the GPU's share */
    int64_t first = 512, cap = kind_shells(kind) == 4 ? 12288 : 262144;
    double growth = 1.25;
    if (const char *e = getenv("CINTGPU_CHUNK")) {   /* "first,growth,cap" (tuning) */
        long long f = 0, c = 0;
        double g = 0;
        if (sscanf(e, "%lld,%lf,%lld", &f, &g, &c) == 3 && f >= 1 && g >= 1.0 && c >= f) {
            first = f; growth = g; cap = c;
        }
    }
    for (int64_t i0 = 0, len = first; i0 < n;
         i0 += len, len = std::min<int64_t>(std::max<int64_t>(len + (growth > 1.0), (int64_t)(len * growth)), cap)) {
        Chunk x;
        x.i0 = i0;
        x.n = std::min(len, n - i0);
        x.base = total;
        for (int64_t q = x.i0; q < x.i0 + x.n; q++) total += item_block(kind, shls + nsh * q, bas);
        ch.push_back(x);
    }
    const int C = (int)ch.size(), R = CG_BATCH_SLOTS;
    std::mutex mu;
    std::condition_variable cv;
    bool abort = false;
    std::atomic<int> next_build{0}, next_scatter{0};
    int dev = 0;
    cudaGetDevice(&dev);
    auto fail = [&](int c, int r, const std::string &e) {
        std::lock_guard<std::mutex> lk(mu);
        if (!abort) { ch[c].rc = r; ch[c].err = e; }
        abort = true;
        cv.notify_all();
    };
    using clk = std::chrono::steady_clock;
    auto since = [](clk::time_point a) { return std::chrono::duration<double, std::milli>(clk::now() - a).count(); };
    const auto t_start = clk::now();
    std::atomic<int64_t> us_build{0}, us_image{0}, us_first{-1};
    auto builder = [&]() {
        cudaSetDevice(dev);   /* the planner queries kernel occupancy on the caller's device */
        for (;;) {
            const int c = next_build.fetch_add(1);
            if (c >= C) return;
            auto tb = clk::now();
            CINTGPUPlan *P = new CINTGPUPlan();
            /* chunks are small: a separate output kernel on the chunk's stream beats transforms at
             * the integral kernel's tail (measured for int2e to host memory and int3c2e to device
             * memory alike) */
            P->fuse_out = false;
            int r = build_plan(P, kind, shls + nsh * ch[c].i0, ch[c].n, nullptr, atm, natm, bas, nbas, env, 0);
            us_build += (int64_t)(1e3 * since(tb));
            if (r) { fail(c, r, cintgpu_last_error()); delete P; return; }
            const int slot = c % R;
            if (c >= R) {   /* the slot's image buffer is free once chunk c - R is uploaded */
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] { return abort || ch[c - R].h2d; });
                if (abort) { delete P; return; }
                lk.unlock();
                if (cudaEventSynchronize(X.ev_h2d[slot]) != cudaSuccess) {
                    fail(c, CINTGPU_ERR_CUDA, "upload failed");
                    delete P;
                    return;
                }
            }
            DevLayout D = dev_layout(P);
            if ((r = grow_host(&X.pin_in[slot], &X.pin_in_cap[slot], D.upload))) {
                fail(c, r, cintgpu_last_error());
                delete P;
                return;
            }
            auto ti = clk::now();
            fill_image(P, D, X.pin_in[slot]);
            us_image += (int64_t)(1e3 * since(ti));
            if (c == 0) us_first = (int64_t)(1e3 * since(t_start));
            std::lock_guard<std::mutex> lk(mu);
            ch[c].P = P;
            ch[c].D = D;
            ch[c].out_size = P->out_size;
            ch[c].ncomp = P->ncomp;
            ch[c].t_ready = since(t_start);
            ch[c].image = true;
            cv.notify_all();
        }
    };
    auto scatter = [&]() {
        for (;;) {
            const int c = next_scatter.fetch_add(1);
            if (c >= C) return;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] { return abort || ch[c].d2h; });
                if (abort) return;
            }
            const int slot = c % R;
            if (cudaEventSynchronize(X.ev_d2h[slot]) != cudaSuccess) {
                fail(c, CINTGPU_ERR_CUDA, "copy back failed");
                return;
            }
            for (int k = 0; k < ch[c].ncomp; k++)
                memcpy(out_host + (size_t)k * total + ch[c].base,
                       X.pin_out[slot] + sizeof(double) * k * ch[c].out_size, sizeof(double) * ch[c].out_size);
            std::lock_guard<std::mutex> lk(mu);
            ch[c].scattered = true;
            cv.notify_all();
        }
    };
    const int nbuild = std::max(1, std::min<int>(C, std::min<int>(14, (int)std::thread::hardware_concurrency())));
    const int nscatter = out_dev ? 0 : std::min(C, 2);
    std::vector<std::thread> pool;
    for (int t = 0; t < nbuild; t++) pool.emplace_back(builder);
    for (int t = 0; t < nscatter; t++) pool.emplace_back(scatter);

    /* CINTGPU_TRACE=1: the caller's time per phase, printed to stderr at the end */
    const bool trace = getenv("CINTGPU_TRACE") != nullptr;
    double t_image = 0, t_slot = 0, t_enqueue = 0;
    for (int c = 0; c < C; c++) {
        const int slot = c % R;
        cudaStream_t st = X.s_exec[slot];
        CINTGPUPlan *P;
        {
            auto t0 = clk::now();
            std::unique_lock<std::mutex> lk(mu);
            cv.wait(lk, [&] { return abort || ch[c].image; });
            t_image += since(t0);
            if (abort) break;
            t0 = clk::now();
            /* slot reuse: chunk c - R copied back and scattered (so its kernels are done too); with
             * device output the slot's stream orders the reuse after that chunk's kernels */
            if (c >= R && !out_dev) cv.wait(lk, [&] { return abort || ch[c - R].scattered; });
            t_slot += since(t0);
            if (abort) break;
            P = ch[c].P;
        }
        auto t0 = clk::now();
        ch[c].t_enq = since(t_start);
        const DevLayout &D = ch[c].D;
        const size_t outb = sizeof(double) * std::max<int64_t>(P->out_size * P->ncomp, 1);
        int r;
        /* device output: the slot's previous chunk may still run from its arena; a growing
         * arena waits for it first */
        if (out_dev && D.total > X.arena_cap[slot] && cudaStreamSynchronize(st) != cudaSuccess) {
            fail(c, CINTGPU_ERR_CUDA, "chunk stream failed");
            break;
        }
        if ((r = grow_dev(&X.arena[slot], &X.arena_cap[slot], D.total))
            || (!out_dev && (r = grow_dev(&X.dout[slot], &X.dout_cap[slot], outb)))
            || (!out_dev && (r = grow_host(&X.pin_out[slot], &X.pin_out_cap[slot], outb)))) {
            fail(c, r, cintgpu_last_error());
            break;
        }
        P->dbuf = X.arena[slot]; P->dbuf_size = X.arena_cap[slot]; P->owns_dbuf = false;
        carve_plan(P, D, X.arena[slot]);
        bool ok = cudaMemcpyAsync(X.arena[slot], X.pin_in[slot], D.upload, cudaMemcpyHostToDevice, st) == cudaSuccess
                  && cudaEventRecord(X.ev_h2d[slot], st) == cudaSuccess;
        if (ok) {
            std::lock_guard<std::mutex> lk(mu);
            ch[c].h2d = true;
            cv.notify_all();
        }
        double *dst = out_dev ? out_dev + ch[c].base : (double *)X.dout[slot];
        if (ok && (r = execute_plan(P, dst, st))) { fail(c, r, cintgpu_last_error()); break; }
        ok = ok && cudaEventRecord(X.ev_exec[slot], st) == cudaSuccess;
        if (!out_dev)
            ok = ok && cudaStreamWaitEvent(X.s_copy, X.ev_exec[slot], 0) == cudaSuccess
                 && cudaMemcpyAsync(X.pin_out[slot], X.dout[slot], outb, cudaMemcpyDeviceToHost, X.s_copy) == cudaSuccess
                 && cudaEventRecord(X.ev_d2h[slot], X.s_copy) == cudaSuccess;
        if (!ok) {
            fail(c, CINTGPU_ERR_CUDA, std::string("chunk enqueue failed: ") + cudaGetErrorString(cudaGetLastError()));
            break;
        }
        {
            std::lock_guard<std::mutex> lk(mu);
            ch[c].d2h = true;
            ch[c].P = nullptr;
            cv.notify_all();
        }
        delete P;   /* its device data live in the slot's arena; the host images are not needed */
        t_enqueue += since(t0);
    }
    for (std::thread &t : pool) t.join();
    for (int s = 0; s < CG_BATCH_SLOTS; s++) cudaStreamSynchronize(X.s_exec[s]);
    cudaStreamSynchronize(X.s_copy);
    for (Chunk &x : ch) {
        delete x.P;
        if (x.rc && !rc) { rc = x.rc; set_error("%s", x.err.c_str()); }
    }
    if (trace)
        fprintf(stderr, "cintgpu_batch_host: %lld items, %d chunks, %d builders; caller ms: waiting for "
                        "images %.1f, waiting for free slots %.1f, enqueue %.1f, total %.1f; builders ms: "
                        "planning %.1f, images %.1f, first image at %.1f\n",
                (long long)n, C, nbuild, t_image, t_slot, t_enqueue, since(t_start), 1e-3 * us_build,
                1e-3 * us_image, 1e-3 * us_first);
    if (trace) {
        fprintf(stderr, "cintgpu_batch_host chunks (items: image ready / enqueued, ms):");
        for (int c = 0; c < C; c++) fprintf(stderr, " %lld:%.1f/%.1f", (long long)ch[c].n, ch[c].t_ready, ch[c].t_enq);
        fprintf(stderr, "\n");
    }
    return rc;
}

/* Whole-molecule J / K / adjoint over a Schwarz-screened quartet list that is never stored
 * (libcint's caller pattern, examples/time_c2h6.c:719-745, with the per-pair bound of its
 * optimizer's pair data, src/optimizer.c:344-425).  The shell pairs are sorted by their bound
 * Q, largest first; the unique quartets are the pairs (p, q) of that order with q <= p and
 * Q_p Q_q >= threshold, so for every bra position p the surviving kets are the prefix
 * [0, min(p + 1, n_p)) with n_p found by binary search.  The quartets of bra positions
 * [p_begin, p_end) are cut into chunks in this order; builder threads materialise each chunk's
 * quartets and build its J / K / adjoint plan (primitive screening as everywhere), the caller
 * uploads and executes the chunk plans on two streams through a ring of four device slots; the
 * contraction accumulates into vj / vk / grad on the device, so no integral is stored.
 * Synchronous: returns when every chunk has run.  *nquartets (may be NULL) receives the number
 * of quartets evaluated. */
static int screened_run(int kind, const int *pairs, const double *q, int64_t npair, double threshold,
                        int64_t p_begin, int64_t p_end, const int *atm, int natm, const int *bas,
                        int nbas, const double *env, const double *dm_dev, double *vj_dev,
                        double *vk_dev, double *grad_dev, double *galpha_dev, int64_t *nquartets)
{
    if (nquartets) *nquartets = 0;
    if (!(kind == CINTGPU_J_BUILD || kind == CINTGPU_K_BUILD || kind == CINTGPU_JK_BUILD
          || kind == CINTGPU_J_GRAD || kind == CINTGPU_J_GRAD_EXP)) {
        set_error("screened runs take the J, K, J+K and adjoint kinds");
        return CINTGPU_ERR_ARG;
    }
    if (npair < 0 || !(threshold >= 0) || !dm_dev) { set_error("bad pair list, threshold or density"); return CINTGPU_ERR_ARG; }
    const bool grad = kind == CINTGPU_J_GRAD || kind == CINTGPU_J_GRAD_EXP;
    if ((grad && !grad_dev) || (kind == CINTGPU_J_GRAD_EXP && !galpha_dev)
        || ((kind == CINTGPU_J_BUILD || kind == CINTGPU_JK_BUILD) && !vj_dev)
        || ((kind == CINTGPU_K_BUILD || kind == CINTGPU_JK_BUILD) && !vk_dev)) {
        set_error("the kind's outputs must be given");
        return CINTGPU_ERR_ARG;
    }
    for (int64_t t = 0; t < npair; t++)
        if (pairs[2 * t] < 0 || pairs[2 * t] >= nbas || pairs[2 * t + 1] < 0 || pairs[2 * t + 1] >= nbas
            || !std::isfinite(q[t])) {
            set_error("pair %lld: shells (%d, %d) outside 0..%d or bound not finite", (long long)t,
                      pairs[2 * t], pairs[2 * t + 1], nbas - 1);
            return CINTGPU_ERR_ARG;
        }
    int rc = ensure_init();
    if (rc) return rc;
    /* order by bound, largest first (stable: equal bounds keep the caller's order) */
    std::vector<int64_t> ord((size_t)npair);
    for (int64_t t = 0; t < npair; t++) ord[t] = t;
    std::stable_sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) { return q[a] > q[b]; });
    std::vector<double> qs((size_t)npair);
    for (int64_t t = 0; t < npair; t++) qs[t] = q[ord[t]];
    p_begin = std::max<int64_t>(0, p_begin);
    p_end = std::min<int64_t>(npair, p_end < 0 ? npair : p_end);
    /* kets of bra position p: [0, kets(p)) */
    auto kets = [&](int64_t p) -> int64_t {
        if (qs[p] <= 0) return 0;
        const double need = threshold / qs[p];
        /* first position whose bound is below need */
        const int64_t n = std::upper_bound(qs.begin(), qs.end(), need,
                                           [](double v, double e) { return v > e; }) - qs.begin();
        /* positions [0, n) have qs >= need only when qs[pos] * qs[p] >= threshold exactly */
        int64_t m = n;
        while (m > 0 && qs[m - 1] * qs[p] < threshold) m--;
        while (m < npair && qs[m] * qs[p] >= threshold) m++;
        return std::min<int64_t>(p + 1, m);
    };
    /* chunks of about `target` quartets along (p, q) */
    struct Span { int64_t p0, q0, p1, q1, n; };   /* from (p0, q0) up to, excluding, (p1, q1) */
    std::vector<Span> spans;
    const int64_t target = grad ? 20000 : 40000;
    int64_t total = 0;
    {
        Span cur{p_begin, 0, p_begin, 0, 0};
        for (int64_t p = p_begin; p < p_end; p++) {
            const int64_t k = kets(p);
            int64_t q0 = 0;
            while (q0 < k) {
                const int64_t take = std::min(k - q0, target - cur.n);
                q0 += take;
                cur.n += take;
                total += take;
                if (cur.n == target) {
                    cur.p1 = p; cur.q1 = q0;
                    spans.push_back(cur);
                    cur = Span{p, q0, p, q0, 0};
                }
            }
        }
        if (cur.n > 0) { cur.p1 = p_end - 1; cur.q1 = kets(p_end - 1); spans.push_back(cur); }
    }
    if (nquartets) *nquartets = total;
    if (spans.empty()) return 0;
    BatchCtx &X = tl_batch;
    rc = X.init();
    if (rc) return rc;
    const int C = (int)spans.size(), R = CG_BATCH_SLOTS;
    struct Chunk { CINTGPUPlan *P = nullptr; DevLayout D; bool image = false, h2d = false, done = false; int rc = 0; std::string err; };
    std::vector<Chunk> ch(C);
    std::mutex mu;
    std::condition_variable cv;
    bool abort = false;
    std::atomic<int> next{0};
    int dev = 0;
    cudaGetDevice(&dev);
    auto fail = [&](int c, int r, const std::string &e) {
        std::lock_guard<std::mutex> lk(mu);
        if (!abort) { ch[c].rc = r; ch[c].err = e; }
        abort = true;
        cv.notify_all();
    };
    auto builder = [&]() {
        cudaSetDevice(dev);
        std::vector<int> items;
        for (;;) {
            const int c = next.fetch_add(1);
            if (c >= C) return;
            const Span &sp = spans[c];
            items.clear();
            items.reserve((size_t)sp.n * 4);
            for (int64_t p = sp.p0; p <= sp.p1 && p < p_end; p++) {
                const int64_t k = kets(p);
                const int64_t qa = p == sp.p0 ? sp.q0 : 0, qb = p == sp.p1 ? std::min(k, sp.q1) : k;
                const int *bra = pairs + 2 * ord[p];
                for (int64_t t = qa; t < qb; t++) {
                    const int *ket = pairs + 2 * ord[t];
                    items.push_back(bra[0]); items.push_back(bra[1]);
                    items.push_back(ket[0]); items.push_back(ket[1]);
                }
            }
            CINTGPUPlan *P = new CINTGPUPlan();
            int r = build_plan(P, kind, items.data(), (int64_t)items.size() / 4, nullptr, atm, natm,
                               bas, nbas, env, 0);
            if (r) { fail(c, r, cintgpu_last_error()); delete P; return; }
            const int slot = c % R;
            if (c >= R) {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] { return abort || ch[c - R].h2d; });
                if (abort) { delete P; return; }
                lk.unlock();
                if (cudaEventSynchronize(X.ev_h2d[slot]) != cudaSuccess) { fail(c, CINTGPU_ERR_CUDA, "upload failed"); delete P; return; }
            }
            DevLayout D = dev_layout(P);
            if ((r = grow_host(&X.pin_in[slot], &X.pin_in_cap[slot], D.upload))) { fail(c, r, cintgpu_last_error()); delete P; return; }
            fill_image(P, D, X.pin_in[slot]);
            std::lock_guard<std::mutex> lk(mu);
            ch[c].P = P;
            ch[c].D = D;
            ch[c].image = true;
            cv.notify_all();
        }
    };
    const int nbuild = std::max(1, std::min<int>(C, std::min<int>(14, (int)std::thread::hardware_concurrency())));
    std::vector<std::thread> pool;
    for (int t = 0; t < nbuild; t++) pool.emplace_back(builder);
    for (int c = 0; c < C; c++) {
        const int slot = c % R;
        cudaStream_t st = X.s_exec[c & 1];
        CINTGPUPlan *P;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv.wait(lk, [&] { return abort || ch[c].image; });
            if (abort) break;
            P = ch[c].P;
        }
        /* the slot's previous chunk must have finished executing before its arena is reused */
        if (c >= R && cudaEventSynchronize(X.ev_exec[slot]) != cudaSuccess) { fail(c, CINTGPU_ERR_CUDA, "chunk execution failed"); break; }
        const DevLayout &D = ch[c].D;
        int r;
        if ((r = grow_dev(&X.arena[slot], &X.arena_cap[slot], D.total))) { fail(c, r, cintgpu_last_error()); break; }
        P->dbuf = X.arena[slot]; P->dbuf_size = X.arena_cap[slot]; P->owns_dbuf = false;
        carve_plan(P, D, X.arena[slot]);
        bool ok = cudaMemcpyAsync(X.arena[slot], X.pin_in[slot], D.upload, cudaMemcpyHostToDevice, st) == cudaSuccess
                  && cudaEventRecord(X.ev_h2d[slot], st) == cudaSuccess;
        if (ok) { std::lock_guard<std::mutex> lk(mu); ch[c].h2d = true; cv.notify_all(); }
        P->cur_dm = dm_dev;
        P->cur_vj = P->jmode & 1 ? vj_dev : nullptr;
        P->cur_vk = P->jmode & 2 ? vk_dev : nullptr;
        P->cur_grad = grad_dev;
        P->cur_galpha = galpha_dev;
        if (ok && (r = execute_plan(P, nullptr, st))) { fail(c, r, cintgpu_last_error()); break; }
        if (!ok || cudaEventRecord(X.ev_exec[slot], st) != cudaSuccess) { fail(c, CINTGPU_ERR_CUDA, "chunk enqueue failed"); break; }
        std::lock_guard<std::mutex> lk(mu);
        ch[c].P = nullptr;
        delete P;
    }
    for (std::thread &t : pool) t.join();
    cudaStreamSynchronize(X.s_exec[0]);
    cudaStreamSynchronize(X.s_exec[1]);
    for (Chunk &x : ch) {
        delete x.P;
        if (x.rc && !rc) { rc = x.rc; set_error("%s", x.err.c_str()); }
    }
    if (!rc && cudaGetLastError() != cudaSuccess) { set_error("screened run failed on the device"); rc = CINTGPU_ERR_CUDA; }
    return rc;
}

int cintgpu_screened_run(int kind, const int *pairs, const double *q, int64_t npair,
                         double threshold, int64_t p_begin, int64_t p_end, const int *atm, int natm,
                         const int *bas, int nbas, const double *env, const double *dm_dev,
                         double *vj_dev, double *vk_dev, double *grad_dev, double *galpha_dev,
                         int64_t *nquartets)
{
    return screened_run(kind, pairs, q, npair, threshold, p_begin, p_end, atm, natm, bas, nbas, env,
                        dm_dev, vj_dev, vk_dev, grad_dev, galpha_dev, nquartets);
}

int cintgpu_batch_device(int kind, double *out_dev, const int *shls, int64_t n, const int *atm,
                         int natm, const int *bas, int nbas, const double *env)
{
    if (kind == CINTGPU_J_BUILD || kind == CINTGPU_K_BUILD || kind == CINTGPU_JK_BUILD
        || kind == CINTGPU_J_GRAD || kind == CINTGPU_J_GRAD_EXP) {
        set_error("cintgpu_batch_device computes integral blocks; J, K and the gradient need a density");
        return CINTGPU_ERR_ARG;
    }
    const int mode_comp = (kind == CINTGPU_INT2E_SPH || kind == CINTGPU_INT2E_CART || kind == CINTGPU_INT3C2E_SPH
                           || kind == CINTGPU_INT3C2E_CART || kind == CINTGPU_INT2C2E_SPH
                           || kind == CINTGPU_INT2C2E_CART) ? 1 : 0;
    if (!mode_comp) {
        set_error("cintgpu_batch_device takes the one-component kinds (int2e, int3c2e, int2c2e)");
        return CINTGPU_ERR_ARG;
    }
    if (!out_dev && n > 0) { set_error("null output"); return CINTGPU_ERR_ARG; }
    if (n <= 0) return 0;
    int rc = ensure_init();
    if (rc) return rc;
    return batch_host_pipelined(kind, nullptr, shls, n, atm, natm, bas, nbas, env, out_dev);
}

int cintgpu_batch_host(int kind, double *out_host, const int *shls, int64_t n,
                       const int64_t *offsets, const int *atm, int natm, const int *bas,
                       int nbas, const double *env)
{
    if (kind == CINTGPU_J_BUILD || kind == CINTGPU_K_BUILD || kind == CINTGPU_JK_BUILD
        || kind == CINTGPU_J_GRAD || kind == CINTGPU_J_GRAD_EXP) {
        set_error("cintgpu_batch_host computes integral blocks; J, K and the gradient need a density "
                  "(cintgpu_plan_execute_jk / cintgpu_plan_execute_grad)");
        return CINTGPU_ERR_ARG;
    }
    if (n <= 0) return 0;
    int rc = ensure_init();
    if (rc) return rc;
    if (!offsets) return batch_host_pipelined(kind, out_host, shls, n, atm, natm, bas, nbas, env);
    CINTGPUPlan *P = nullptr;
    rc = cintgpu_plan_create(&P, kind, shls, n, offsets, atm, natm, bas, nbas, env);
    if (rc) return rc;
    size_t outb = sizeof(double) * P->out_size * P->ncomp;
    double *dout = nullptr;
    if (cudaMalloc(&dout, std::max<size_t>(outb, 8)) != cudaSuccess) {
        set_error("cudaMalloc(%zu) failed", outb);
        cintgpu_plan_destroy(P);
        return CINTGPU_ERR_NOMEM;
    }
    if (offsets) cudaMemcpy(dout, out_host, outb, cudaMemcpyHostToDevice);
    rc = execute_plan(P, dout, 0);
    if (!rc && cudaMemcpy(out_host, dout, outb, cudaMemcpyDeviceToHost) != cudaSuccess) {
        set_error("device to host copy failed: %s", cudaGetErrorString(cudaGetLastError()));
        rc = CINTGPU_ERR_CUDA;
    }
    cudaFree(dout);
    cintgpu_plan_destroy(P);
    return rc;
}

/* ---- libcint drop-in ---------------------------------------------------------------------- */
CACHE_SIZE_T int2e_sph(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm, FINT *bas,
                       FINT nbas, double *env, CINTOpt *opt, double *cache)
{ (void)cache; return dropin(CINTGPU_INT2E_SPH, out, dims, shls, atm, natm, bas, nbas, env, opt); }
CACHE_SIZE_T int2e_cart(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm, FINT *bas,
                        FINT nbas, double *env, CINTOpt *opt, double *cache)
{ (void)cache; return dropin(CINTGPU_INT2E_CART, out, dims, shls, atm, natm, bas, nbas, env, opt); }
CACHE_SIZE_T int2e_ip1_sph(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm, FINT *bas,
                           FINT nbas, double *env, CINTOpt *opt, double *cache)
{ (void)cache; return dropin(CINTGPU_INT2E_IP1_SPH, out, dims, shls, atm, natm, bas, nbas, env, opt); }
CACHE_SIZE_T int2e_ip1_cart(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm, FINT *bas,
                            FINT nbas, double *env, CINTOpt *opt, double *cache)
{ (void)cache; return dropin(CINTGPU_INT2E_IP1_CART, out, dims, shls, atm, natm, bas, nbas, env, opt); }
CACHE_SIZE_T int2e_ip2_sph(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm, FINT *bas,
                           FINT nbas, double *env, CINTOpt *opt, double *cache)
{ (void)cache; return dropin(CINTGPU_INT2E_IP2_SPH, out, dims, shls, atm, natm, bas, nbas, env, opt); }
CACHE_SIZE_T int2e_ip2_cart(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm, FINT *bas,
                            FINT nbas, double *env, CINTOpt *opt, double *cache)
{ (void)cache; return dropin(CINTGPU_INT2E_IP2_CART, out, dims, shls, atm, natm, bas, nbas, env, opt); }
CACHE_SIZE_T int2e_ipip1_sph(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm, FINT *bas,
                             FINT nbas, double *env, CINTOpt *opt, double *cache)
{ (void)cache; return dropin(CINTGPU_INT2E_IPIP1_SPH, out, dims, shls, atm, natm, bas, nbas, env, opt); }
CACHE_SIZE_T int2e_ipip1_cart(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm, FINT *bas,
                              FINT nbas, double *env, CINTOpt *opt, double *cache)
{ (void)cache; return dropin(CINTGPU_INT2E_IPIP1_CART, out, dims, shls, atm, natm, bas, nbas, env, opt); }
CACHE_SIZE_T int3c2e_ip1_sph(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm, FINT *bas,
                             FINT nbas, double *env, CINTOpt *opt, double *cache)
{ (void)cache; return dropin(CINTGPU_INT3C2E_IP1_SPH, out, dims, shls, atm, natm, bas, nbas, env, opt); }
CACHE_SIZE_T int3c2e_ip1_cart(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm, FINT *bas,
                              FINT nbas, double *env, CINTOpt *opt, double *cache)
{ (void)cache; return dropin(CINTGPU_INT3C2E_IP1_CART, out, dims, shls, atm, natm, bas, nbas, env, opt); }
CACHE_SIZE_T int3c2e_ip2_sph(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm, FINT *bas,
                             FINT nbas, double *env, CINTOpt *opt, double *cache)
{ (void)cache; return dropin(CINTGPU_INT3C2E_IP2_SPH, out, dims, shls, atm, natm, bas, nbas, env, opt); }
CACHE_SIZE_T int3c2e_ip2_cart(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm, FINT *bas,
                              FINT nbas, double *env, CINTOpt *opt, double *cache)
{ (void)cache; return dropin(CINTGPU_INT3C2E_IP2_CART, out, dims, shls, atm, natm, bas, nbas, env, opt); }
CACHE_SIZE_T int3c2e_sph(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm, FINT *bas,
                         FINT nbas, double *env, CINTOpt *opt, double *cache)
{ (void)cache; return dropin(CINTGPU_INT3C2E_SPH, out, dims, shls, atm, natm, bas, nbas, env, opt); }
CACHE_SIZE_T int3c2e_cart(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm, FINT *bas,
                          FINT nbas, double *env, CINTOpt *opt, double *cache)
{ (void)cache; return dropin(CINTGPU_INT3C2E_CART, out, dims, shls, atm, natm, bas, nbas, env, opt); }
CACHE_SIZE_T int2c2e_sph(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm, FINT *bas,
                         FINT nbas, double *env, CINTOpt *opt, double *cache)
{ (void)cache; return dropin(CINTGPU_INT2C2E_SPH, out, dims, shls, atm, natm, bas, nbas, env, opt); }
CACHE_SIZE_T int2c2e_cart(double *out, FINT *dims, FINT *shls, FINT *atm, FINT natm, FINT *bas,
                          FINT nbas, double *env, CINTOpt *opt, double *cache)
{ (void)cache; return dropin(CINTGPU_INT2C2E_CART, out, dims, shls, atm, natm, bas, nbas, env, opt); }

/* The optimizer keeps libcint's CINTOpt layout; its content is the side table above (the shell
 * pairs' primitive data, built on first use by the drop-in calls made with it). */
void int2e_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env)
{ (void)atm; (void)natm; (void)bas; (void)env; make_opt(opt, nbas); }
void int2e_ip1_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env)
{ (void)atm; (void)natm; (void)bas; (void)env; make_opt(opt, nbas); }
void int3c2e_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env)
{ (void)atm; (void)natm; (void)bas; (void)env; make_opt(opt, nbas); }
void int2c2e_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env)
{ (void)atm; (void)natm; (void)bas; (void)env; make_opt(opt, nbas); }
void int2e_ip2_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env)
{ (void)atm; (void)natm; (void)bas; (void)env; make_opt(opt, nbas); }
void int3c2e_ip1_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env)
{ (void)atm; (void)natm; (void)bas; (void)env; make_opt(opt, nbas); }
void int2e_ipip1_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env)
{ (void)atm; (void)natm; (void)bas; (void)env; make_opt(opt, nbas); }
void int3c2e_ip2_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env)
{ (void)atm; (void)natm; (void)bas; (void)env; make_opt(opt, nbas); }
void CINTdel_2e_optimizer(CINTOpt **opt)
{
    if (opt && *opt) {
        {
            std::lock_guard<std::mutex> lk(g_opt_mu);
            g_opt_states.erase(*opt);
        }
        free(*opt);
        *opt = NULL;
    }
}
void CINTdel_optimizer(CINTOpt **opt) { CINTdel_2e_optimizer(opt); }

FINT cint2e_sph(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env, CINTOpt *opt)
{ return int2e_sph(out, NULL, shls, atm, natm, bas, nbas, env, opt, NULL); }
FINT cint2e_cart(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env, CINTOpt *opt)
{ return int2e_cart(out, NULL, shls, atm, natm, bas, nbas, env, opt, NULL); }
void cint2e_sph_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env)
{ int2e_optimizer(opt, atm, natm, bas, nbas, env); }
void cint2e_cart_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env)
{ int2e_optimizer(opt, atm, natm, bas, nbas, env); }
FINT cint2e_ip1_sph(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env, CINTOpt *opt)
{ return int2e_ip1_sph(out, NULL, shls, atm, natm, bas, nbas, env, opt, NULL); }
FINT cint2e_ip1_cart(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env, CINTOpt *opt)
{ return int2e_ip1_cart(out, NULL, shls, atm, natm, bas, nbas, env, opt, NULL); }
void cint2e_ip1_sph_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env)
{ int2e_ip1_optimizer(opt, atm, natm, bas, nbas, env); }
FINT cint2e_ip2_sph(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env, CINTOpt *opt)
{ return int2e_ip2_sph(out, NULL, shls, atm, natm, bas, nbas, env, opt, NULL); }
FINT cint2e_ip2_cart(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env, CINTOpt *opt)
{ return int2e_ip2_cart(out, NULL, shls, atm, natm, bas, nbas, env, opt, NULL); }
void cint2e_ip2_sph_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env)
{ int2e_ip2_optimizer(opt, atm, natm, bas, nbas, env); }
FINT cint2e_ipip1_sph(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env, CINTOpt *opt)
{ return int2e_ipip1_sph(out, NULL, shls, atm, natm, bas, nbas, env, opt, NULL); }
FINT cint2e_ipip1_cart(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env, CINTOpt *opt)
{ return int2e_ipip1_cart(out, NULL, shls, atm, natm, bas, nbas, env, opt, NULL); }
void cint2e_ipip1_sph_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env)
{ int2e_ipip1_optimizer(opt, atm, natm, bas, nbas, env); }
FINT cint3c2e_ip1_sph(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env, CINTOpt *opt)
{ return int3c2e_ip1_sph(out, NULL, shls, atm, natm, bas, nbas, env, opt, NULL); }
FINT cint3c2e_ip1_cart(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env, CINTOpt *opt)
{ return int3c2e_ip1_cart(out, NULL, shls, atm, natm, bas, nbas, env, opt, NULL); }
FINT cint3c2e_ip2_sph(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env, CINTOpt *opt)
{ return int3c2e_ip2_sph(out, NULL, shls, atm, natm, bas, nbas, env, opt, NULL); }
FINT cint3c2e_ip2_cart(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env, CINTOpt *opt)
{ return int3c2e_ip2_cart(out, NULL, shls, atm, natm, bas, nbas, env, opt, NULL); }
FINT cint3c2e_sph(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env, CINTOpt *opt)
{ return int3c2e_sph(out, NULL, shls, atm, natm, bas, nbas, env, opt, NULL); }
FINT cint3c2e_cart(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env, CINTOpt *opt)
{ return int3c2e_cart(out, NULL, shls, atm, natm, bas, nbas, env, opt, NULL); }
void cint3c2e_sph_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env)
{ int3c2e_optimizer(opt, atm, natm, bas, nbas, env); }
FINT cint2c2e_sph(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env, CINTOpt *opt)
{ return int2c2e_sph(out, NULL, shls, atm, natm, bas, nbas, env, opt, NULL); }
FINT cint2c2e_cart(double *out, FINT *shls, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env, CINTOpt *opt)
{ return int2c2e_cart(out, NULL, shls, atm, natm, bas, nbas, env, opt, NULL); }
void cint2c2e_sph_optimizer(CINTOpt **opt, FINT *atm, FINT natm, FINT *bas, FINT nbas, double *env)
{ int2c2e_optimizer(opt, atm, natm, bas, nbas, env); }

/* ---- basis helpers (libcint src/misc.c:72-93, src/cint_bas.c) ------------------------------ */
double CINTgto_norm(FINT n, double a)
{
    /* 1/sqrt(int_0^inf r^(2n+2) exp(-2 a r^2) dr) */
    double n1 = (2 * n + 2 + 1) * .5;
    double gi = exp(lgamma(n1)) / (2. * pow(2 * a, n1));
    return 1. / sqrt(gi);
}
FINT CINTlen_cart(const FINT l) { return (l + 1) * (l + 2) / 2; }
FINT CINTcgto_cart(const FINT bas_id, const FINT *bas)
{ const FINT *b = bas + BAS_SLOTS * bas_id; return ncart_l(b[ANG_OF]) * b[NCTR_OF]; }
FINT CINTcgto_spheric(const FINT bas_id, const FINT *bas)
{ const FINT *b = bas + BAS_SLOTS * bas_id; return nsph_l(b[ANG_OF]) * b[NCTR_OF]; }
FINT CINTtot_cgto_cart(const FINT *bas, const FINT nbas)
{ FINT s = 0; for (FINT i = 0; i < nbas; i++) s += CINTcgto_cart(i, bas); return s; }
FINT CINTtot_cgto_spheric(const FINT *bas, const FINT nbas)
{ FINT s = 0; for (FINT i = 0; i < nbas; i++) s += CINTcgto_spheric(i, bas); return s; }
void CINTshells_cart_offset(FINT ao_loc[], const FINT *bas, const FINT nbas)
{ ao_loc[0] = 0; for (FINT i = 1; i < nbas; i++) ao_loc[i] = ao_loc[i - 1] + CINTcgto_cart(i - 1, bas); }
void CINTshells_spheric_offset(FINT ao_loc[], const FINT *bas, const FINT nbas)
{ ao_loc[0] = 0; for (FINT i = 1; i < nbas; i++) ao_loc[i] = ao_loc[i - 1] + CINTcgto_spheric(i - 1, bas); }

}  /* extern "C" */

/* ================================================================== internal hooks */
#include "cintgpu_internal.h"

int cg_init(void) { return ensure_init(); }
int cg_sm_count(void) { return g_ctx.sm_count; }
void cg_set_error_msg(const char *msg) { set_error("%s", msg); }
/* Contraction-first tables of one class (bra = 1: the bra-per-term tables), for host-side tests
 * of the table logic: info[12] = CGEriClass fields, groups[4 * ngroup], perm[nE + nF], prog (the transfer program),
 * rounds[nround]; returns the program length or -1 when a buffer is too small. */
extern "C" int cg_eri_tables(int li, int lj, int lk, int ll, int bra, int *info, int *groups,
                             int maxg, int *perm, int maxp, int *prog, int maxprog, int *rounds,
                             int maxr)
{
    CINTGPUPlan P;
    build_eri_class(&P, li, lj, lk, ll, bra != 0);
    const CGEriClass &c = P.eclass[0];
    if (c.ngroup > maxg || c.nE + c.nF > maxp || (int)P.hprog.size() > maxprog || c.nround > maxr) return -1;
    memcpy(info, &c, sizeof(CGEriClass));
    memcpy(groups, P.egroup.data(), sizeof(CGEriGroup) * P.egroup.size());
    memcpy(perm, P.eperm.data(), sizeof(int) * P.eperm.size());
    memcpy(prog, P.hprog.data(), sizeof(int) * P.hprog.size());
    memcpy(rounds, P.eround.data(), sizeof(int) * P.eround.size());
    return (int)P.hprog.size();
}

/* tasks of a built plan whose class transfers the bra per term */
static int64_t bra_tasks(const CINTGPUPlan &P)
{
    int64_t n = 0;
    for (int g = 0; g < 2; g++)
        for (int t = P.groups[g].task0; t < P.groups[g].task0 + P.groups[g].ntasks; t++)
            n += P.eclass.empty() ? 0 : P.eclass[P.tasks[t].cls].bra;
    return n;
}

/* Host planning only, for tests of the task routing: info[0..2] = tasks of the three groups
 * (regular, 48 KB, per-primitive int2e), info[3] = 1 when outputs are transformed inside the
 * integral kernel, info[4] = tasks of classes transferring the bra per term. */
extern "C" int cg_plan_groups(int kind, const int *shls, int64_t n, const int *atm, int natm,
                              const int *bas, int nbas, const double *env, int64_t *info)
{
    CINTGPUPlan P;
    int rc = build_plan(&P, kind, shls, n, nullptr, atm, natm, bas, nbas, env, 0);
    if (rc) return rc;
    for (int g = 0; g < 3; g++) info[g] = P.groups[g].ntasks;
    info[3] = fused(&P) ? 1 : 0;
    info[4] = P.mode == CG_MODE_ERI ? bra_tasks(P) : 0;
    return 0;
}

/* the groups with classes forced into the 48 KB group (per-class tuning) */
extern "C" int cg_plan_groups_wide(int kind, const int *shls, int64_t n, const int *atm, int natm,
                                   const int *bas, int nbas, const double *env, const int *wide,
                                   int nwide, int64_t *info)
{
    CINTGPUPlan P;
    if (nwide > 0) P.wide.assign(wide, wide + nwide);
    int rc = build_plan(&P, kind, shls, n, nullptr, atm, natm, bas, nbas, env, 0);
    if (rc) return rc;
    for (int g = 0; g < 3; g++) info[g] = P.groups[g].ntasks;
    return 0;
}

/* the same with the regular group's shared memory per warp set (KB); info[4] = that group's
 * doubles per warp */
extern "C" int cg_plan_groups_ws(int kind, const int *shls, int64_t n, const int *atm, int natm,
                                 const int *bas, int nbas, const double *env, int ws_kb,
                                 int64_t *info)
{
    CINTGPUPlan P;
    P.ws_kb = ws_kb;
    int rc = build_plan(&P, kind, shls, n, nullptr, atm, natm, bas, nbas, env, 0);
    if (rc) return rc;
    for (int g = 0; g < 3; g++) info[g] = P.groups[g].ntasks;
    info[3] = fused(&P) ? 1 : 0;
    info[4] = P.groups[0].ws;
    return 0;
}

/* Test hook: FNV-1a hash of a host-built plan's upload image, its launch groups and the scalars
 * its executions read, so that changes to the planner can be checked to produce identical plans. */
extern "C" int cg_plan_image_hash(int kind, const int *shls, int64_t n, const int *atm, int natm,
                                  const int *bas, int nbas, const double *env, int64_t split_target,
                                  uint64_t *hash)
{
    CINTGPUPlan P;
    P.plan_threads = (int)std::thread::hardware_concurrency();
    int rc = build_plan(&P, kind, shls, n, nullptr, atm, natm, bas, nbas, env, split_target);
    if (rc) return rc;
    DevLayout D = dev_layout(&P);
    std::vector<char> img(D.upload);
    fill_image(&P, D, img.data());
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](const void *p, size_t len) {
        const unsigned char *c = (const unsigned char *)p;
        for (size_t i = 0; i < len; i++) { h ^= c[i]; h *= 1099511628211ull; }
    };
    mix(img.data(), img.size());
    for (int g = 0; g < 3; g++) {
        const TaskGroup &G = P.groups[g];
        int v[5] = {G.task0, G.ntasks, G.ws, G.blocks_per_sm, G.nblocks};
        mix(v, sizeof(v));
    }
    int64_t s[8] = {P.out_size, P.max_nf, P.hrr_max, P.nef_max, P.prim_quartets, P.nao_cart,
                    (int64_t)P.fuse_out, (int64_t)P.empty_outs.size()};
    mix(s, sizeof(s));
    double f[2] = {P.flops, P.flops_ref};
    mix(f, sizeof(f));
    *hash = h;
    return 0;
}

CINTGPUPlan *cg_plan_new(void) { return new CINTGPUPlan(); }
void cg_plan_separate_output(CINTGPUPlan *P) { P->fuse_out = false; }
void cg_plan_free_host(CINTGPUPlan *P) { P->dbuf = nullptr; delete P; }

int cg_plan_build(CINTGPUPlan *P, int kind, const int *shls, int64_t n, const int64_t *offsets,
                  const int *atm, int natm, const int *bas, int nbas, const double *env,
                  int64_t split_target)
{
    return build_plan(P, kind, shls, n, offsets, atm, natm, bas, nbas, env, split_target);
}

size_t cg_plan_bytes(const CINTGPUPlan *P) { return plan_device_bytes(P); }

int cg_plan_place(CINTGPUPlan *P, char *region, size_t region_bytes, cudaStream_t stream)
{
    DevLayout D = dev_layout(P);
    if (D.total > region_bytes) { set_error("plan needs %zu bytes, region has %zu", D.total, region_bytes); return CINTGPU_ERR_NOMEM; }
    P->dbuf = region; P->dbuf_size = region_bytes; P->owns_dbuf = false;
    carve_plan(P, D, region);
    std::vector<char> img(D.upload);
    fill_image(P, D, img.data());
    /* pageable source: returns once the data is staged, so img may be released afterwards */
    CUDA_OK(cudaMemcpyAsync(region, img.data(), D.upload, cudaMemcpyHostToDevice, stream));
    return 0;
}

int cg_plan_run(CINTGPUPlan *P, double *out_dev, cudaStream_t stream)
{
    return execute_plan(P, out_dev, stream);
}
