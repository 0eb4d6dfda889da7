// hcore-gb300 — batched plan API (include/hcore_gb300.h) and shared host
// helpers for the drop-in entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "hc_host.h"

namespace hc {

static thread_local std::string g_last_error;

void set_error(const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

const char *last_error() { return g_last_error.c_str(); }

// Device-accessible alias of p: device/managed memory as is, pinned host
// memory through its device pointer; pageable host memory yields nullptr.
const void *device_alias(const void *p) {
    if (!p) return nullptr;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    switch (at.type) {
        case cudaMemoryTypeDevice:
        case cudaMemoryTypeManaged:
            return p;
        case cudaMemoryTypeHost:
            return at.devicePointer ? at.devicePointer : p;
        default:
            return nullptr;
    }
}

bool is_device_memory(const void *p) {
    if (!p) return false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// Validate one task and fill its descriptor; returns the task status
// (0 = runnable).  Mirrors the reference's exit(-1) conditions, in the order
// HCORE_dgemm checks them.
int fill_desc(const hcore_lr_task &t, unsigned flags, bool translate, Desc &d, int &k_out) {
    memset(&d, 0, sizeof d);
    const bool fast = flags & HCORE_GPU_FAST_RULES;
    const int a = t.a, b = t.b, c = t.c, M = t.M;
    const int k = a + c;
    k_out = k > 0 ? k : 0;
    d.M = M;
    d.a = a;
    d.b = b;
    d.c = c;
    d.k = k_out;
    d.alpha = t.alpha;
    d.beta = t.beta;
    d.acc = t.acc;
    d.rk = t.rk;
    d.lda = t.lda;
    d.ldb = t.ldb;
    d.ldc = t.ldc;
    d.ldco = t.ldco;
    d.rank_start = fast ? 2 : 1;
    d.max_rank = fast ? INT_MAX : t.maxrk;
    d.storage_rank = t.storage_maxrank > 0 ? t.storage_maxrank : INT_MAX;
    if (a < 0 || b < 0 || c < 0 || M < 1) return HCORE_GPU_S_SHAPE;
    if (k == 0) return HCORE_GPU_S_ZERO_RANK;
    if (!fast && k > 2 * t.maxrk) return HCORE_GPU_S_RANK_SUM;
    const int ld_newv = t.ld_newv > 0 ? t.ld_newv : 2 * t.maxrk;
    if (!fast && ld_newv < k) return HCORE_GPU_S_LDNEWV;
    if (k > M || k > kMaxK || M > 32 * kMaxRowsPerLane) return HCORE_GPU_S_SHAPE;
    if ((a > 0 && t.lda < M) || (b > 0 && t.ldb < M && !t.Bdense) || (c > 0 && t.ldc < M) ||
        t.ldco < M)
        return HCORE_GPU_S_SHAPE;
    auto tr = [&](const void *p) { return translate ? device_alias(p) : p; };
    d.AU = a ? tr(t.AU) : nullptr;
    d.AV = a ? tr(t.AV) : nullptr;
    if (t.Bdense) {
        d.Bd = a ? tr(t.Bdense) : nullptr;
        if (a && !d.Bd) return HCORE_GPU_S_SHAPE;
    } else {
        d.BU = (a && b) ? tr(t.BU) : nullptr;
        d.BV = (a && b) ? tr(t.BV) : nullptr;
        if (a && b && (!d.BU || !d.BV)) return HCORE_GPU_S_SHAPE;
    }
    d.CU = c ? tr(t.CU) : nullptr;
    d.CV = c ? tr(t.CV) : nullptr;
    d.CUo = const_cast<void *>(tr(t.CUo));
    d.CVo = const_cast<void *>(tr(t.CVo));
    if ((a && (!d.AU || !d.AV)) || (c && (!d.CU || !d.CV)) || !d.CUo || !d.CVo)
        return HCORE_GPU_S_SHAPE;
    return HCORE_GPU_S_OK;
}

// Build the descriptors of a batch, sorted by decreasing k (then cost) so that
// the long updates start first (longest-processing-time order) and the rank
// buckets are contiguous; rejected tasks go last.
void fill_buckets(const std::vector<Desc> &descs, LaunchShape &shape) {
    shape.nbuckets = 0;
    const int n = (int)descs.size();
    int i = 0;
    while (i < n) {
        const int w = shape.bucket_width;
        const int K = descs[i].status0 ? bucket_edge(1, w) : bucket_edge(descs[i].k, w);
        int j = i;
        while (j < n && (descs[j].status0 ? bucket_edge(1, w) : bucket_edge(descs[j].k, w)) == K) ++j;
        if (shape.nbuckets == kMaxBuckets) {  // cannot happen with the fixed edges; merge
            shape.buckets[kMaxBuckets - 1].count += j - i;
        } else {
            shape.buckets[shape.nbuckets++] = Bucket{i, j - i, K};
        }
        i = j;
    }
    // the rebuild launch is sized for the most columns an accepted update
    // can have (a predicted capacity passed as storage_maxrank shrinks it)
    shape.maxR = 1;
    for (const Desc &d : descs)
        if (!d.status0) shape.maxR = std::max(shape.maxR, std::min(d.k, d.storage_rank));
    // each launch is sized for the largest k actually present in its bucket
    for (int b = 0; b < shape.nbuckets; ++b) {
        int K = 1;
        const Bucket &bk = shape.buckets[b];
        for (int x = bk.start; x < bk.start + bk.count; ++x)
            if (!descs[x].status0) K = std::max(K, descs[x].k);
        shape.buckets[b].K = K;
    }
}

bool build_descs(int n, const hcore_lr_task *tasks, unsigned flags, bool translate,
                 std::vector<Desc> &descs, long long &ws_elems, int &maxM, int &maxK,
                 std::vector<int> *status0) {
    descs.resize(n);
    std::vector<double> cost(n);
    maxM = 1;
    maxK = 1;
    for (int i = 0; i < n; ++i) {
        int k = 0;
        const int st = fill_desc(tasks[i], flags, translate, descs[i], k);
        descs[i].status0 = st;
        descs[i].idx = i;
        if (status0) (*status0)[i] = st;
        cost[i] = st ? -1.0 : (double)k * 1e12 + (double)tasks[i].M * k * k;
        if (!st) {
            maxM = std::max(maxM, tasks[i].M);
            maxK = std::max(maxK, k);
        }
    }
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost[x] > cost[y]; });
    std::vector<Desc> sorted(n);
    long long off = 0;
    for (int j = 0; j < n; ++j) {
        Desc d = descs[order[j]];
        d.ws = off;
        if (!d.status0) off += ws_layout(d).total;
        sorted[j] = d;
    }
    descs.swap(sorted);
    ws_elems = off;
    return true;
}

}  // namespace hc

using namespace hc;

struct hcore_gpu_plan_s {
    int prec = 0;
    int n = 0;
    unsigned flags = 0;
    int maxM = 1, maxK = 1;
    LaunchShape shape;  // of the whole plan when it runs as one group
    // stream groups: the sorted updates are dealt round-robin into groups,
    // each launched on its own stream so that one group's latency-bound SVD
    // CTAs share the SMs with another group's FP64-bound QR/rebuild CTAs
    struct Group {
        int start = 0, count = 0;
        LaunchShape shape;
        cudaStream_t stream = nullptr;
        cudaEvent_t done = nullptr;
    };
    std::vector<Group> groups;
    cudaEvent_t gfork = nullptr;
    Desc *d_desc = nullptr;
    int *d_rank = nullptr;
    int *d_status = nullptr;
    int *d_info = nullptr;  // Jacobi sweeps per task
    void *d_ws = nullptr;
    size_t ws_bytes = 0;
    std::vector<long long> ws_of_task;
    std::vector<int> k_of_task;
    std::vector<Desc> h_desc;        // host copy of d_desc (launch order)
    std::vector<int> pos_of_task;    // task index -> position in h_desc
    Desc *d_rdesc = nullptr;         // hcore_gpu_plan_rebuild: descriptors and indices
    int *d_ridx = nullptr;
    int rcap = 0;
    // HCORE_GPU_STAGE_INPUTS: host input ranges merged into segments, each
    // mirrored in d_mirror and refreshed by one copy per execute
    struct Segment {
        const char *host;
        size_t bytes, off;
    };
    std::vector<Segment> segs;
    char *d_mirror = nullptr;
    size_t staged_bytes = 0;
    size_t zero_copy_bytes = 0;   // pinned host inputs read in place by the kernels
    // some task's output overlaps another task's input: the stream groups
    // finish every stack phase before any later phase starts
    bool cross_alias = false;
    bool phase_sync = false;   // tuning: all groups finish each phase before the next
    std::vector<cudaEvent_t> stacked;   // per group, with cross_alias
};

namespace {

// Does an output range of one task overlap an input range of another?  (A
// task's own C may be updated in place: its inputs are read in the stack
// phase, before its rebuild writes.)  Ranges are conservative: every output
// of M x max(c, a + c) columns.
bool outputs_alias_other_inputs(int n, const hcore_lr_task *tasks, size_t esz) {
    struct Rng {
        const char *lo, *hi;
        int task;
        bool out;
    };
    std::vector<Rng> rr;
    auto add = [&](const void *ptr, int rows, int ld, int ncol, int task, bool out) {
        if (!ptr || ncol <= 0 || rows <= 0) return;
        const char *lo = (const char *)ptr;
        rr.push_back({lo, lo + ((size_t)(ncol - 1) * ld + rows) * esz, task, out});
    };
    for (int q = 0; q < n; ++q) {
        const hcore_lr_task &t = tasks[q];
        if (t.a > 0) {
            add(t.AU, t.M, t.lda, t.a, q, false);
            add(t.AV, t.M, t.lda, t.a, q, false);
        }
        if (t.Bdense) add(t.Bdense, t.M, t.ldb, t.M, q, false);
        else if (t.b > 0) {
            add(t.BU, t.M, t.ldb, t.b, q, false);
            add(t.BV, t.M, t.ldb, t.b, q, false);
        }
        if (t.c > 0) {
            add(t.CU, t.M, t.ldc, t.c, q, false);
            add(t.CV, t.M, t.ldc, t.c, q, false);
        }
        const int ncol = std::max(t.c, t.a + t.c);
        add(t.CUo, t.M, t.ldco, ncol, q, true);
        add(t.CVo, t.M, t.ldco, ncol, q, true);
    }
    std::sort(rr.begin(), rr.end(), [](const Rng &x, const Rng &y) { return x.lo < y.lo; });
    // sweep: every range against the ranges still open at its start
    std::vector<const Rng *> open;
    for (const Rng &r : rr) {
        size_t w = 0;
        for (const Rng *o : open)
            if (o->hi > r.lo) open[w++] = o;
        open.resize(w);
        for (const Rng *o : open)
            if (o->task != r.task && (o->out != r.out || (o->out && r.out))) return true;
        open.push_back(&r);
    }
    return false;
}

// Host inputs of a plan with HCORE_GPU_STAGE_INPUTS.  A host range that
// several updates read (a panel tile), or that lies in pageable memory, is
// mirrored on the device and refreshed by one copy per merged segment at the
// start of every execute; the tasks' pointers are replaced by their mirror
// addresses.  A pinned range read by one update only (its own C tile) is
// left in place: the stack kernel reads it over the host link once, as a
// copy would, but while other stream groups compute.  Returns false on
// allocation failure.
bool stage_inputs(hcore_gpu_plan p, std::vector<hcore_lr_task> &tt, size_t esz) {
    struct Rng {
        const char *lo, *hi;
        int task;
        bool pinned;
    };
    std::vector<Rng> rr;
    int cur = 0;
    auto add = [&](const void *ptr, int rows, int ld, int ncol) {
        if (!ptr || ncol <= 0 || rows <= 0) return;
        cudaPointerAttributes at;
        bool pinned = false;
        if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess) {
            cudaGetLastError();                       // unknown to CUDA: pageable host memory
        } else if (at.type == cudaMemoryTypeHost) {
            pinned = at.devicePointer != nullptr;
        } else if (at.type != cudaMemoryTypeUnregistered) {
            return;                                   // device or managed memory: used in place
        }
        const char *lo = (const char *)ptr;
        rr.push_back({lo, lo + ((size_t)(ncol - 1) * ld + rows) * esz, cur, pinned});
    };
    for (size_t q = 0; q < tt.size(); ++q) {
        const hcore_lr_task &t = tt[q];
        cur = (int)q;
        if (t.a > 0) {
            add(t.AU, t.M, t.lda, t.a);
            add(t.AV, t.M, t.lda, t.a);
        }
        if (t.Bdense) add(t.Bdense, t.M, t.ldb, t.M);
        else if (t.b > 0) {
            add(t.BU, t.M, t.ldb, t.b);
            add(t.BV, t.M, t.ldb, t.b);
        }
        if (t.c > 0) {
            add(t.CU, t.M, t.ldc, t.c);
            add(t.CV, t.M, t.ldc, t.c);
        }
    }
    p->staged_bytes = 0;
    p->zero_copy_bytes = 0;
    if (rr.empty()) return true;
    std::sort(rr.begin(), rr.end(), [](const Rng &x, const Rng &y) { return x.lo < y.lo; });
    // clusters of overlapping ranges: staged when read by two or more tasks
    // or not pinned; then adjacent staged clusters merge into segments
    struct Cluster {
        const char *lo, *hi;
        int task;
        bool multi, pinned;
    };
    std::vector<Cluster> cl;
    for (const Rng &r : rr) {
        if (!cl.empty() && r.lo < cl.back().hi) {
            Cluster &c = cl.back();
            c.hi = std::max(c.hi, r.hi);
            c.multi = c.multi || r.task != c.task;
            c.pinned = c.pinned && r.pinned;
        } else {
            cl.push_back({r.lo, r.hi, r.task, false, r.pinned});
        }
    }
    struct Span {
        const char *lo, *hi;
    };
    std::vector<Span> merged;
    for (const Cluster &c : cl) {
        if (!c.multi && c.pinned) {
            p->zero_copy_bytes += (size_t)(c.hi - c.lo);
            continue;
        }
        if (!merged.empty() && c.lo <= merged.back().hi)
            merged.back().hi = std::max(merged.back().hi, c.hi);
        else
            merged.push_back({c.lo, c.hi});
    }
    size_t off = 0;
    for (const Span &m : merged) {
        p->segs.push_back({m.lo, (size_t)(m.hi - m.lo), off});
        off += ((size_t)(m.hi - m.lo) + 255) & ~(size_t)255;
    }
    for (const auto &sg : p->segs) p->staged_bytes += sg.bytes;
    if (p->segs.empty()) return true;
    if (cudaMalloc(&p->d_mirror, off) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    // translate: the segment holding each host pointer (binary search)
    auto tr = [&](const void *ptr) -> const void * {
        if (!ptr) return ptr;
        const char *c = (const char *)ptr;
        size_t lo = 0, hi = p->segs.size();
        while (hi - lo > 1) {
            const size_t mid = (lo + hi) / 2;
            if (p->segs[mid].host <= c) lo = mid;
            else hi = mid;
        }
        const auto &sg = p->segs[lo];
        if (c < sg.host || c >= sg.host + sg.bytes) return ptr;   // not staged: read in place
        return p->d_mirror + sg.off + (size_t)(c - sg.host);
    };
    for (hcore_lr_task &t : tt) {
        if (t.a > 0) {
            t.AU = tr(t.AU);
            t.AV = tr(t.AV);
        }
        if (t.Bdense) t.Bdense = tr(t.Bdense);
        else if (t.b > 0) {
            t.BU = tr(t.BU);
            t.BV = tr(t.BV);
        }
        if (t.c > 0) {
            t.CU = tr(t.CU);
            t.CV = tr(t.CV);
        }
    }
    return true;
}
}  // namespace

static void plan_free(hcore_gpu_plan p) {
    if (!p) return;
    for (int b = 0; b < kMaxBuckets; ++b) {
        if (p->shape.side[b]) cudaStreamDestroy(p->shape.side[b]);
        if (p->shape.join[b]) cudaEventDestroy(p->shape.join[b]);
    }
    if (p->shape.fork) cudaEventDestroy(p->shape.fork);
    for (auto &g : p->groups) {
        if (g.stream) cudaStreamDestroy(g.stream);
        if (g.done) cudaEventDestroy(g.done);
        for (int b = 0; b < kMaxBuckets; ++b) {
            if (g.shape.side[b]) cudaStreamDestroy(g.shape.side[b]);
            if (g.shape.join[b]) cudaEventDestroy(g.shape.join[b]);
        }
        if (g.shape.fork) cudaEventDestroy(g.shape.fork);
    }
    if (p->gfork) cudaEventDestroy(p->gfork);
    for (cudaEvent_t ev : p->stacked)
        if (ev) cudaEventDestroy(ev);
    cudaFree(p->d_desc);
    cudaFree(p->d_rank);
    cudaFree(p->d_status);
    cudaFree(p->d_info);
    cudaFree(p->d_ws);
    cudaFree(p->d_mirror);
    cudaFree(p->d_rdesc);
    cudaFree(p->d_ridx);
    delete p;
}

extern "C" int hcore_gpu_tuning_default(hcore_gpu_tuning *t) {
    if (!t) {
        set_error("hcore_gpu_tuning_default: null argument");
        return HCORE_GPU_EINVAL;
    }
    t->stream_groups = 16;
    if (const char *env = getenv("HCORE_GPU_STREAMS")) t->stream_groups = atoi(env);
    t->stream_groups = std::max(1, std::min(t->stream_groups, 64));
    t->svd_lanes[0] = 2;   // the autotuner's pick on a TLR panel of 1953 updates
    t->svd_lanes[1] = 2;
    t->svd_lanes[2] = 2;
    t->bucket_width = 8;
    t->phase_sync = 0;
    t->qr_warps = 4;
    return HCORE_GPU_OK;
}

static bool valid_tuning(const hcore_gpu_tuning &t) {
    auto lanes = [](int x) { return x == 0 || (x >= 1 && x <= 32 && (x & (x - 1)) == 0); };
    return t.stream_groups >= 1 && t.stream_groups <= 64 && lanes(t.svd_lanes[0]) &&
           lanes(t.svd_lanes[1]) && lanes(t.svd_lanes[2]) &&
           (t.bucket_width == 8 || t.bucket_width == 16) && (t.phase_sync == 0 || t.phase_sync == 1) &&
           (t.qr_warps == 2 || t.qr_warps == 4 || t.qr_warps == 8);
}

extern "C" int hcore_gpu_plan_create(hcore_gpu_plan *plan, int precision, int n,
                                     const hcore_lr_task *tasks, unsigned flags) {
    return hcore_gpu_plan_create_tuned(plan, precision, n, tasks, flags, nullptr);
}

extern "C" int hcore_gpu_plan_create_tuned(hcore_gpu_plan *plan, int precision, int n,
                                           const hcore_lr_task *tasks, unsigned flags,
                                           const hcore_gpu_tuning *tuning) {
    if (!plan || n < 0 || (n > 0 && !tasks) ||
        (precision != HCORE_GPU_F64 && precision != HCORE_GPU_F32)) {
        set_error("hcore_gpu_plan_create: invalid argument");
        return HCORE_GPU_EINVAL;
    }
    hcore_gpu_tuning tune;
    hcore_gpu_tuning_default(&tune);
    if (tuning) {
        if (!valid_tuning(*tuning)) {
            set_error("hcore_gpu_plan_create: invalid tuning (groups 1..64, lanes powers of two "
                      "<= 32, bucket width 8 or 16, phase sync 0 or 1, QR warps 2, 4 or 8)");
            return HCORE_GPU_EINVAL;
        }
        tune = *tuning;
    }
    *plan = nullptr;
    auto *p = new hcore_gpu_plan_s;
    p->prec = precision;
    p->n = n;
    p->flags = flags;
    std::vector<Desc> descs;
    long long ws_elems = 0;
    std::vector<hcore_lr_task> staged;
    if ((flags & HCORE_GPU_STAGE_INPUTS) && n > 0) {
        staged.assign(tasks, tasks + n);
        if (!stage_inputs(p, staged, precision == HCORE_GPU_F64 ? sizeof(double) : sizeof(float))) {
            set_error("hcore_gpu_plan_create: cannot allocate the input mirror");
            plan_free(p);
            return HCORE_GPU_ENOMEM;
        }
        tasks = staged.data();
    }
    p->cross_alias = n > 1 && outputs_alias_other_inputs(
                                  n, tasks, precision == HCORE_GPU_F64 ? sizeof(double) : sizeof(float));
    build_descs(n, tasks, flags, true, descs, ws_elems, p->maxM, p->maxK, nullptr);
    // stream groups (HCORE_GPU_STREAMS, default 16): deal the k-sorted
    // descriptors round-robin so every group gets the same mix of sizes
    int ngroups = std::max(1, std::min(tune.stream_groups, n > 0 ? n : 1));
    p->phase_sync = tune.phase_sync != 0;
    auto set_shape_tuning = [&](LaunchShape &sh) {
        for (int q = 0; q < 3; ++q) sh.svd_lanes[q] = tune.svd_lanes[q];
        sh.bucket_width = tune.bucket_width;
        sh.qr_warps = tune.qr_warps;
    };
    set_shape_tuning(p->shape);
    if (ngroups > 1) {
        std::vector<Desc> dealt;
        dealt.reserve(n);
        for (int g = 0; g < ngroups; ++g) {
            hcore_gpu_plan_s::Group grp;
            grp.start = (int)dealt.size();
            for (int i = g; i < n; i += ngroups) dealt.push_back(descs[i]);
            grp.count = (int)dealt.size() - grp.start;
            p->groups.push_back(grp);
        }
        descs.swap(dealt);
        bool ok = cudaEventCreateWithFlags(&p->gfork, cudaEventDisableTiming) == cudaSuccess;
        for (auto &g : p->groups) {
            std::vector<Desc> sub(descs.begin() + g.start, descs.begin() + g.start + g.count);
            set_shape_tuning(g.shape);
            fill_buckets(sub, g.shape);
            g.shape.maxM = p->maxM;
            g.shape.maxK = p->maxK;
            ok = ok && cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking) == cudaSuccess &&
                 cudaEventCreateWithFlags(&g.done, cudaEventDisableTiming) == cudaSuccess;
            // the group's SVD buckets run concurrently too
            if (ok && g.shape.nbuckets > 1) {
                ok = cudaEventCreateWithFlags(&g.shape.fork, cudaEventDisableTiming) == cudaSuccess;
                for (int b = 0; ok && b < g.shape.nbuckets; ++b)
                    ok = cudaStreamCreateWithFlags(&g.shape.side[b], cudaStreamNonBlocking) ==
                             cudaSuccess &&
                         cudaEventCreateWithFlags(&g.shape.join[b], cudaEventDisableTiming) ==
                             cudaSuccess;
            }
        }
        if (ok && p->cross_alias) {
            p->stacked.assign(p->groups.size(), nullptr);
            for (auto &ev : p->stacked)
                ok = ok && cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess;
        }
        if (!ok) {
            set_error("hcore_gpu_plan_create: cannot create group streams");
            plan_free(p);
            return HCORE_GPU_ECUDA;
        }
    } else {
        fill_buckets(descs, p->shape);
        p->shape.maxM = p->maxM;
        p->shape.maxK = p->maxK;
        if (p->shape.nbuckets > 1) {
            bool ok = cudaEventCreateWithFlags(&p->shape.fork, cudaEventDisableTiming) == cudaSuccess;
            for (int b = 0; ok && b < p->shape.nbuckets; ++b)
                ok = cudaStreamCreateWithFlags(&p->shape.side[b], cudaStreamNonBlocking) ==
                         cudaSuccess &&
                     cudaEventCreateWithFlags(&p->shape.join[b], cudaEventDisableTiming) == cudaSuccess;
            if (!ok) {
                set_error("hcore_gpu_plan_create: cannot create bucket streams");
                plan_free(p);
                return HCORE_GPU_ECUDA;
            }
        }
    }
    p->ws_of_task.assign(n, -1);
    p->k_of_task.assign(n, 0);
    p->pos_of_task.assign(n, -1);
    for (size_t q = 0; q < descs.size(); ++q) {
        const Desc &d = descs[q];
        p->ws_of_task[d.idx] = d.status0 ? -1 : d.ws;
        p->k_of_task[d.idx] = d.k;
        p->pos_of_task[d.idx] = (int)q;
    }
    p->h_desc = descs;
    {
        const cudaError_t ce = precision == HCORE_GPU_F64
                                   ? configure_recompress<double>(p->maxK, &p->shape.svd_smem_kmax,
                                                                  &p->shape.svd_half_kmax)
                                   : configure_recompress<float>(p->maxK, &p->shape.svd_smem_kmax,
                                                                 &p->shape.svd_half_kmax);
        for (auto &g : p->groups) {
            g.shape.svd_smem_kmax = p->shape.svd_smem_kmax;
            g.shape.svd_half_kmax = p->shape.svd_half_kmax;
        }
        const bool mixed = (flags & HCORE_GPU_MIXED_FACTORS) && precision == HCORE_GPU_F64;
        const bool tcr = !(flags & HCORE_GPU_DFMA_REBUILD);
        const bool tcq = !(flags & HCORE_GPU_UNBLOCKED_QR);
        const bool tcs = (flags & HCORE_GPU_TC_STACK) != 0;
        p->shape.mixed = mixed;
        p->shape.tc_rebuild = tcr;
        p->shape.tc_qr = tcq;
        p->shape.tc_stack = tcs;
        for (auto &g : p->groups) {
            g.shape.mixed = mixed;
            g.shape.tc_rebuild = tcr;
            g.shape.tc_qr = tcq;
            g.shape.tc_stack = tcs;
        }
        if (ce != cudaSuccess) {
            set_error("hcore_gpu_plan_create: %s", cudaGetErrorString(ce));
            plan_free(p);
            return HCORE_GPU_ECUDA;
        }
    }
    const size_t esz = precision == HCORE_GPU_F64 ? sizeof(double) : sizeof(float);
    p->ws_bytes = (size_t)ws_elems * esz;
    const size_t nn = (size_t)(n > 0 ? n : 1);
    cudaError_t e = cudaMalloc(&p->d_desc, nn * sizeof(Desc));
    if (e == cudaSuccess) e = cudaMalloc(&p->d_rank, nn * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&p->d_status, nn * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&p->d_info, nn * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&p->d_ws, p->ws_bytes > 0 ? p->ws_bytes : 256);
    if (e != cudaSuccess) {
        set_error("hcore_gpu_plan_create: cudaMalloc failed (%s), workspace %zu bytes",
                  cudaGetErrorString(e), p->ws_bytes);
        cudaGetLastError();
        plan_free(p);
        return HCORE_GPU_ENOMEM;
    }
    if (n > 0) {
        e = cudaMemcpy(p->d_desc, descs.data(), n * sizeof(Desc), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemset(p->d_rank, 0, n * sizeof(int));
        if (e == cudaSuccess) e = cudaMemset(p->d_status, 0, n * sizeof(int));
        if (e == cudaSuccess) e = cudaMemset(p->d_info, 0, n * sizeof(int));
    }
    if (e != cudaSuccess) {
        set_error("hcore_gpu_plan_create: %s", cudaGetErrorString(e));
        plan_free(p);
        return HCORE_GPU_ECUDA;
    }
    *plan = p;
    return HCORE_GPU_OK;
}

extern "C" int hcore_gpu_plan_execute_phases(hcore_gpu_plan p, void *stream, unsigned phases) {
    if (!p) {
        set_error("hcore_gpu_plan_execute: null plan");
        return HCORE_GPU_EINVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSuccess;
    if (phases & kPhaseStack)
        for (const auto &sg : p->segs) {
            e = cudaMemcpyAsync(p->d_mirror + sg.off, sg.host, sg.bytes, cudaMemcpyHostToDevice, s);
            if (e != cudaSuccess) {
                set_error("hcore_gpu_plan_execute: staging copy failed: %s", cudaGetErrorString(e));
                return HCORE_GPU_ECUDA;
            }
        }
    auto launch = [&](const Desc *dd, int cnt, const LaunchShape &sh, cudaStream_t st,
                      unsigned ph) {
        return p->prec == HCORE_GPU_F64
                   ? launch_recompress<double>(dd, cnt, (double *)p->d_ws, p->d_rank, p->d_status,
                                               p->d_info, sh, st, ph & kPhaseAll)
                   : launch_recompress<float>(dd, cnt, (float *)p->d_ws, p->d_rank, p->d_status,
                                              p->d_info, sh, st, ph & kPhaseAll);
    };
    if (p->groups.empty()) {
        e = launch(p->d_desc, p->n, p->shape, s, phases);
    } else if (p->phase_sync) {
        // every group finishes a phase before any group starts the next
        const unsigned order[4] = {kPhaseStack, kPhaseQR, kPhaseSVD, kPhaseApply};
        for (int q = 0; q < 4 && e == cudaSuccess; ++q) {
            const unsigned ph = phases & order[q];
            if (!ph) continue;
            e = cudaEventRecord(p->gfork, s);
            for (auto &g : p->groups) {
                if (e != cudaSuccess) break;
                e = cudaStreamWaitEvent(g.stream, p->gfork, 0);
                if (e == cudaSuccess && g.count > 0)
                    e = launch(p->d_desc + g.start, g.count, g.shape, g.stream, ph);
                if (e == cudaSuccess) e = cudaEventRecord(g.done, g.stream);
                if (e == cudaSuccess) e = cudaStreamWaitEvent(s, g.done, 0);
            }
        }
    } else if (p->cross_alias) {
        // an output of one task overlaps another task's input: every group's
        // stack phase (which reads all inputs) completes before any group
        // goes on to the phases that write outputs
        const size_t ng = p->groups.size();
        e = cudaEventRecord(p->gfork, s);
        for (size_t gi = 0; gi < ng && e == cudaSuccess; ++gi) {
            auto &g = p->groups[gi];
            e = cudaStreamWaitEvent(g.stream, p->gfork, 0);
            if (e == cudaSuccess && g.count > 0)
                e = launch(p->d_desc + g.start, g.count, g.shape, g.stream, phases & kPhaseStack);
            if (e == cudaSuccess) e = cudaEventRecord(p->stacked[gi], g.stream);
        }
        for (size_t gi = 0; gi < ng && e == cudaSuccess; ++gi) {
            auto &g = p->groups[gi];
            for (size_t o = 0; o < ng && e == cudaSuccess; ++o)
                if (o != gi) e = cudaStreamWaitEvent(g.stream, p->stacked[o], 0);
            if (e == cudaSuccess && g.count > 0)
                e = launch(p->d_desc + g.start, g.count, g.shape, g.stream, phases & ~kPhaseStack);
            if (e == cudaSuccess) e = cudaEventRecord(g.done, g.stream);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(s, g.done, 0);
        }
    } else {
        e = cudaEventRecord(p->gfork, s);
        for (auto &g : p->groups) {
            if (e != cudaSuccess) break;
            e = cudaStreamWaitEvent(g.stream, p->gfork, 0);
            if (e == cudaSuccess && g.count > 0)
                e = launch(p->d_desc + g.start, g.count, g.shape, g.stream, phases);
            if (e == cudaSuccess) e = cudaEventRecord(g.done, g.stream);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(s, g.done, 0);
        }
    }
    if (e != cudaSuccess) {
        set_error("hcore_gpu_plan_execute: %s", cudaGetErrorString(e));
        return HCORE_GPU_ECUDA;
    }
    return HCORE_GPU_OK;
}

extern "C" int hcore_gpu_plan_rebuild(hcore_gpu_plan p, int n, const int *task_idx,
                                      void *const *CUo, void *const *CVo, const int *ldco,
                                      const int *max_rank, void *stream) {
    if (!p || n < 0 || (n > 0 && (!task_idx || !CUo || !CVo || !ldco))) {
        set_error("hcore_gpu_plan_rebuild: invalid argument");
        return HCORE_GPU_EINVAL;
    }
    if (n == 0) return HCORE_GPU_OK;
    std::vector<Desc> sub(n);
    int maxM = 1, maxK = 1;
    for (int q = 0; q < n; ++q) {
        const int i = task_idx[q];
        if (i < 0 || i >= p->n || p->pos_of_task[i] < 0 || p->h_desc[p->pos_of_task[i]].status0) {
            set_error("hcore_gpu_plan_rebuild: task %d was not run by this plan", i);
            return HCORE_GPU_EINVAL;
        }
        Desc d = p->h_desc[p->pos_of_task[i]];
        if (!CUo[q] || !CVo[q] || ldco[q] < d.M) {
            set_error("hcore_gpu_plan_rebuild: bad output storage for task %d", i);
            return HCORE_GPU_EINVAL;
        }
        d.CUo = const_cast<void *>(device_alias(CUo[q]));
        d.CVo = const_cast<void *>(device_alias(CVo[q]));
        d.ldco = ldco[q];
        d.storage_rank = INT_MAX;
        sub[q] = d;
        maxM = std::max(maxM, d.M);
        maxK = std::max(maxK, d.k);
    }
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSuccess;
    if (n > p->rcap) {
        cudaFree(p->d_rdesc);
        cudaFree(p->d_ridx);
        p->d_rdesc = nullptr;
        p->d_ridx = nullptr;
        p->rcap = 0;
        e = cudaMalloc(&p->d_rdesc, (size_t)n * sizeof(Desc));
        if (e == cudaSuccess) e = cudaMalloc(&p->d_ridx, 2 * (size_t)n * sizeof(int));
        if (e != cudaSuccess) {
            set_error("hcore_gpu_plan_rebuild: cudaMalloc: %s", cudaGetErrorString(e));
            cudaGetLastError();
            return HCORE_GPU_ENOMEM;
        }
        p->rcap = n;
    }
    // from pageable host memory: both copies are complete when they return
    e = cudaMemcpyAsync(p->d_rdesc, sub.data(), (size_t)n * sizeof(Desc), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(p->d_ridx, task_idx, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && max_rank)
        e = cudaMemcpyAsync(p->d_ridx + n, max_rank, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) {
        const bool mixed = p->shape.mixed;
        const int *cap = max_rank ? p->d_ridx + n : nullptr;
        const bool tcr = p->shape.tc_rebuild;
        e = p->prec == HCORE_GPU_F64
                ? launch_rebuild<double>(p->d_rdesc, p->d_ridx, cap, n, (double *)p->d_ws,
                                         p->d_rank, p->d_status, maxM, maxK, mixed, tcr, s)
                : launch_rebuild<float>(p->d_rdesc, p->d_ridx, cap, n, (float *)p->d_ws,
                                        p->d_rank, p->d_status, maxM, maxK, mixed, tcr, s);
    }
    if (e != cudaSuccess) {
        set_error("hcore_gpu_plan_rebuild: %s", cudaGetErrorString(e));
        return HCORE_GPU_ECUDA;
    }
    return HCORE_GPU_OK;
}

extern "C" int hcore_gpu_plan_execute(hcore_gpu_plan p, void *stream) {
    return hcore_gpu_plan_execute_phases(p, stream, kPhaseAll);
}

extern "C" const int *hcore_gpu_plan_device_ranks(hcore_gpu_plan p) {
    return p ? p->d_rank : nullptr;
}
extern "C" const int *hcore_gpu_plan_device_status(hcore_gpu_plan p) {
    return p ? p->d_status : nullptr;
}
extern "C" int hcore_gpu_plan_sweeps(hcore_gpu_plan p, int *sweeps, void *stream) {
    if (!p || !sweeps) {
        set_error("hcore_gpu_plan_sweeps: invalid argument");
        return HCORE_GPU_EINVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSuccess;
    if (p->n) e = cudaMemcpyAsync(sweeps, p->d_info, p->n * sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_error("hcore_gpu_plan_sweeps: %s", cudaGetErrorString(e));
        return HCORE_GPU_ECUDA;
    }
    return HCORE_GPU_OK;
}

extern "C" int hcore_gpu_plan_launches(hcore_gpu_plan p) {
    if (!p || p->n == 0) return 0;
    const bool fp64 = p->prec == HCORE_GPU_F64;
    auto count = [fp64](const LaunchShape &sh) {
        // stack (and its tensor-core products), QR, SVD buckets, rebuild
        int c = 1 + (fp64 && sh.tc_stack && !sh.mixed) + qr_launches(sh, fp64) +
                rebuild_launches(sh, fp64);
        for (int b = 0; b < sh.nbuckets; ++b) c += sh.buckets[b].count > 0;
        return c;
    };
    if (p->groups.empty()) return count(p->shape);
    int c = 0;
    for (const auto &g : p->groups)
        if (g.count > 0) c += count(g.shape);
    return c;
}

extern "C" size_t hcore_gpu_plan_workspace_bytes(hcore_gpu_plan p) { return p ? p->ws_bytes : 0; }
extern "C" size_t hcore_gpu_plan_staged_bytes(hcore_gpu_plan p) { return p ? p->staged_bytes : 0; }
extern "C" size_t hcore_gpu_plan_zero_copy_bytes(hcore_gpu_plan p) {
    return p ? p->zero_copy_bytes : 0;
}

extern "C" int hcore_gpu_plan_results(hcore_gpu_plan p, int *ranks, int *status, void *stream) {
    if (!p) {
        set_error("hcore_gpu_plan_results: null plan");
        return HCORE_GPU_EINVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaSuccess;
    if (ranks && p->n)
        e = cudaMemcpyAsync(ranks, p->d_rank, p->n * sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && status && p->n)
        e = cudaMemcpyAsync(status, p->d_status, p->n * sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_error("hcore_gpu_plan_results: %s", cudaGetErrorString(e));
        return HCORE_GPU_ECUDA;
    }
    if (status)
        for (int i = 0; i < p->n; ++i)
            if (status[i]) return HCORE_GPU_ETASK;
    return HCORE_GPU_OK;
}

extern "C" int hcore_gpu_plan_sigma(hcore_gpu_plan p, int i, double *sigma, int *k, void *stream) {
    if (!p || i < 0 || i >= p->n) {
        set_error("hcore_gpu_plan_sigma: invalid argument");
        return HCORE_GPU_EINVAL;
    }
    const int kk = p->k_of_task[i];
    if (k) *k = kk;
    if (!sigma || p->ws_of_task[i] < 0 || kk == 0) return HCORE_GPU_OK;
    // task i's descriptor holds its layout; recompute the sigma offset
    std::vector<Desc> one(1);
    cudaStream_t s = (cudaStream_t)stream;
    // locate the descriptor of task i
    std::vector<Desc> all(p->n);
    cudaError_t e = cudaMemcpy(all.data(), p->d_desc, p->n * sizeof(Desc), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        set_error("hcore_gpu_plan_sigma: %s", cudaGetErrorString(e));
        return HCORE_GPU_ECUDA;
    }
    for (const Desc &d : all)
        if (d.idx == i) one[0] = d;
    const WsLayout L = ws_layout(one[0]);
    const long long off = one[0].ws + L.sig;
    if (p->prec == HCORE_GPU_F64) {
        e = cudaMemcpyAsync(sigma, (double *)p->d_ws + off, kk * sizeof(double),
                            cudaMemcpyDeviceToHost, s);
    } else {
        std::vector<float> tmp(kk);
        e = cudaMemcpyAsync(tmp.data(), (float *)p->d_ws + off, kk * sizeof(float),
                            cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        for (int j = 0; j < kk; ++j) sigma[j] = tmp[j];
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_error("hcore_gpu_plan_sigma: %s", cudaGetErrorString(e));
        return HCORE_GPU_ECUDA;
    }
    return HCORE_GPU_OK;
}

extern "C" int hcore_gpu_plan_destroy(hcore_gpu_plan p) {
    plan_free(p);
    return HCORE_GPU_OK;
}

static int batched_once(int prec, int n, const hcore_lr_task *tasks, int *ranks, int *status,
                        void *stream) {
    hcore_gpu_plan p = nullptr;
    int rc = hcore_gpu_plan_create(&p, prec, n, tasks, 0);
    if (rc) return rc;
    rc = hcore_gpu_plan_execute(p, stream);
    if (!rc) rc = hcore_gpu_plan_results(p, ranks, status, stream);
    hcore_gpu_plan_destroy(p);
    return rc;
}

extern "C" int hcore_gpu_dgemm_batched(int n, const hcore_lr_task *tasks, int *ranks, int *status,
                                       void *stream) {
    return batched_once(HCORE_GPU_F64, n, tasks, ranks, status, stream);
}

extern "C" int hcore_gpu_sgemm_batched(int n, const hcore_lr_task *tasks, int *ranks, int *status,
                                       void *stream) {
    return batched_once(HCORE_GPU_F32, n, tasks, ranks, status, stream);
}

extern "C" const char *hcore_gpu_last_error(void) { return last_error(); }
extern "C" int hcore_gpu_version(void) { return 100; }

// ---------------------------------------------------------------------------
// autotuner: coordinate descent over the launch-shape parameters, timing
// plans of the caller's own batch
// ---------------------------------------------------------------------------
extern "C" int hcore_gpu_autotune(int precision, int n, const hcore_lr_task *tasks, unsigned flags,
                                  int reps, void *stream, hcore_gpu_tuning *best, double *best_ms) {
    if (n <= 0 || !tasks || !best) {
        set_error("hcore_gpu_autotune: invalid argument");
        return HCORE_GPU_EINVAL;
    }
    reps = std::max(1, reps);
    cudaStream_t s = (cudaStream_t)stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        set_error("hcore_gpu_autotune: cannot create events");
        if (e0) cudaEventDestroy(e0);
        return HCORE_GPU_ECUDA;
    }
    // A candidate is timed the way a plan is meant to run: its execute
    // captured once in a CUDA graph and the graph replayed (launch overhead
    // then hardly depends on the number of launches).  A plan that cannot be
    // captured (pageable staged inputs) is timed by direct executes.
    cudaStream_t cs = nullptr;
    if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        set_error("hcore_gpu_autotune: cannot create a stream");
        return HCORE_GPU_ECUDA;
    }
    (void)s;
    auto time_cfg = [&](const hcore_gpu_tuning &t, double &ms) -> int {
        hcore_gpu_plan p = nullptr;
        int rc = hcore_gpu_plan_create_tuned(&p, precision, n, tasks, flags, &t);
        if (rc) return rc;
        rc = hcore_gpu_plan_execute(p, cs);   // warm-up
        cudaError_t e = rc ? cudaSuccess : cudaStreamSynchronize(cs);
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ge = nullptr;
        if (!rc && e == cudaSuccess) {
            bool captured = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
            if (captured) {
                const int xrc = hcore_gpu_plan_execute(p, cs);
                captured = cudaStreamEndCapture(cs, &g) == cudaSuccess && xrc == 0 &&
                           cudaGraphInstantiate(&ge, g, 0) == cudaSuccess;
            }
            if (!captured) {
                cudaGetLastError();
                if (ge) cudaGraphExecDestroy(ge);
                if (g) cudaGraphDestroy(g);
                ge = nullptr;
                g = nullptr;
            }
        }
        auto run_once = [&]() -> int {
            if (ge) return cudaGraphLaunch(ge, cs) == cudaSuccess ? 0 : HCORE_GPU_ECUDA;
            return hcore_gpu_plan_execute(p, cs);
        };
        if (!rc && e == cudaSuccess && ge) e = cudaGraphUpload(ge, cs);   // no extra execute
        if (!rc && e == cudaSuccess) e = cudaStreamSynchronize(cs);
        if (!rc && e == cudaSuccess) e = cudaEventRecord(e0, cs);
        for (int r = 0; r < reps && !rc && e == cudaSuccess; ++r) rc = run_once();
        if (!rc && e == cudaSuccess) e = cudaEventRecord(e1, cs);
        if (!rc && e == cudaSuccess) e = cudaEventSynchronize(e1);
        float f = 0.f;
        if (!rc && e == cudaSuccess) e = cudaEventElapsedTime(&f, e0, e1);
        if (ge) cudaGraphExecDestroy(ge);
        if (g) cudaGraphDestroy(g);
        hcore_gpu_plan_destroy(p);
        if (!rc && e != cudaSuccess) {
            set_error("hcore_gpu_autotune: %s", cudaGetErrorString(e));
            rc = HCORE_GPU_ECUDA;
        }
        ms = (double)f / reps;
        return rc;
    };
    hcore_gpu_tuning cur;
    hcore_gpu_tuning_default(&cur);
    double cur_ms = 0;
    int rc = time_cfg(cur, cur_ms);
    // one parameter at a time, keeping a change only if it gains 0.5 %
    const int groups[] = {4, 8, 16, 24, 32};
    const int lanes0[] = {0, 1, 2}, lanes1[] = {0, 1, 2, 4, 8}, lanes2[] = {0, 1, 2, 4};
    const int widths[] = {8, 16};
    // field(t) is the parameter being searched, as a reference into t
    auto try_values = [&](auto field, const int *vals, int nv) {
        for (int v = 0; v < nv && !rc; ++v) {
            if (vals[v] == field(cur)) continue;
            hcore_gpu_tuning t = cur;
            field(t) = vals[v];
            double ms = 0;
            rc = time_cfg(t, ms);
            if (!rc && ms < cur_ms * 0.995) {
                cur = t;
                cur_ms = ms;
            }
        }
    };
    const int syncs[] = {0, 1};
    try_values([](hcore_gpu_tuning &t) -> int & { return t.phase_sync; }, syncs, 2);
    try_values([](hcore_gpu_tuning &t) -> int & { return t.stream_groups; }, groups, 5);
    const int qrw[] = {8, 4, 2};
    try_values([](hcore_gpu_tuning &t) -> int & { return t.qr_warps; }, qrw, 3);
    try_values([](hcore_gpu_tuning &t) -> int & { return t.svd_lanes[1]; }, lanes1, 5);
    try_values([](hcore_gpu_tuning &t) -> int & { return t.svd_lanes[2]; }, lanes2, 4);
    try_values([](hcore_gpu_tuning &t) -> int & { return t.svd_lanes[0]; }, lanes0, 3);
    try_values([](hcore_gpu_tuning &t) -> int & { return t.bucket_width; }, widths, 2);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(cs);
    if (rc) return rc;
    *best = cur;
    if (best_ms) *best_ms = cur_ms;
    return HCORE_GPU_OK;
}
