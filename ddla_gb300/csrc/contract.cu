// Two-operand einsum (MArray.Contract) lowered to batched GEMM.
//
// Plan (host): the index analysis of DDLA's MArray.Contract
// (DDLA/Einsum/MArray.Contract.cs:48-125, IndiceUtils.Diagonal/Divide/Fold,
// DDLA/Utilities/IndiceUtils.cs:18-245): repeated symbols become one mode with
// summed strides; modes split into batch (in A, B and C, then C-only, A-only,
// B-only), M (A and C), N (B and C), K (A and B); contiguous M/N/K modes fold;
// M and N sort by descending C stride, K by descending A stride; operands swap
// when N's innermost C stride is 1.
//
// Execution (device): each (M, N, K) triple that folds to one mode each is a
// strided GEMM C += alpha A B run as one batched DMMA launch over the batch
// modes that write distinct C elements (an offset table per batch index).
// Batch modes that sum into the same C (A-only / B-only modes, C stride 0)
// run as sequential launches so no two concurrent tiles update the same C.
// Multi-mode M / N / K go through a gather into dense operands, the same GEMM,
// and a scatter-add back (DDLA's BlockScatterMatrix plays this role,
// DDLA/Einsum/BlockScatterMatrix.cs:205-324).
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"
#include "timing.cuh"

namespace ddla {

int gemm_f64_offsets(cudaStream_t s, i64 m, i64 n, i64 k, double alpha, View<const double> A,
                     View<const double> B, double beta, View<double> C, i64 batch, const i64 *d_offsets);
int gemm_ozaki(ddla_handle h, i64 m, i64 n, i64 k, double alpha, View<const double> A, View<const double> B,
               double beta, View<double> C, int uplo = DDLA_DENSE, i64 batch = 1,
               const i64 *d_offsets = nullptr);

namespace {

struct Ent {
    char sym;
    i64 len, stride;
    bool used;
};

int diagonal(const std::string &sym, int rank, const i64 *len, const i64 *str, std::vector<Ent> &out) {
    out.clear();
    if ((int)sym.size() != rank) return -1;
    for (int i = 0; i < rank; i++) {
        auto it = std::find_if(out.begin(), out.end(), [&](const Ent &e) { return e.sym == sym[i]; });
        if (it != out.end()) {
            if (it->len != len[i]) return -1;
            it->stride += str[i];
        } else {
            out.push_back(Ent{sym[i], len[i], str[i], false});
        }
    }
    return 0;
}

i64 field(const ddla_contract_mode &m, int f) { return f == 0 ? m.sa : (f == 1 ? m.sb : m.sc); }

// Outer mode absorbs an inner one when both strides equal len*stride of the
// inner one (IndiceUtils.Fold, DoubleIndices variant).
void fold2(std::vector<ddla_contract_mode> &v, int f1, int f2) {
    bool changed = true;
    while (changed) {
        changed = false;
        for (size_t o = 0; o < v.size() && !changed; o++)
            for (size_t in = 0; in < v.size() && !changed; in++) {
                if (o == in) continue;
                if (field(v[o], f1) == v[in].len * field(v[in], f1) && field(v[o], f2) == v[in].len * field(v[in], f2)) {
                    v[o].len *= v[in].len;
                    v[o].sa = v[in].sa;
                    v[o].sb = v[in].sb;
                    v[o].sc = v[in].sc;
                    v.erase(v.begin() + in);
                    changed = true;
                }
            }
    }
}

void sort_desc(std::vector<ddla_contract_mode> &v, int f) {
    std::stable_sort(v.begin(), v.end(),
                     [&](const ddla_contract_mode &x, const ddla_contract_mode &y) { return field(x, f) > field(y, f); });
}

i64 total(const ddla_contract_mode *v, int n) {
    i64 t = 1;
    for (int i = 0; i < n; i++) t *= v[i].len;
    return t;
}

// Offsets of every flattened index of a mode list (last mode fastest).
std::vector<i64> offsets(const ddla_contract_mode *v, int n, int f) {
    i64 tot = total(v, n);
    std::vector<i64> out((size_t)tot);
    for (i64 x = 0; x < tot; x++) {
        i64 rem = x, off = 0;
        for (int i = n - 1; i >= 0; i--) {
            i64 idx = rem % v[i].len;
            rem /= v[i].len;
            off += idx * field(v[i], f);
        }
        out[(size_t)x] = off;
    }
    return out;
}

// dense[i*ld + j] = src[rowoff[i] + coloff[j]]
__global__ void k_gather(const double *src, const i64 *rowoff, const i64 *coloff, i64 rows, i64 cols, double *dst) {
    i64 tot = rows * cols;
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
        i64 i = e / cols, j = e % cols;
        dst[e] = src[rowoff[i] + coloff[j]];
    }
}
// dst[rowoff[i] + coloff[j]] += dense[i*cols + j]  (distinct targets within one call)
__global__ void k_scatter_add(const double *dense, const i64 *rowoff, const i64 *coloff, i64 rows, i64 cols,
                              double *dst) {
    i64 tot = rows * cols;
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < tot; e += (i64)gridDim.x * blockDim.x) {
        i64 i = e / cols, j = e % cols;
        dst[rowoff[i] + coloff[j]] += dense[e];
    }
}

int grid_of(i64 tot) {
    i64 g = (tot + 255) / 256;
    return (int)(g < 1 ? 1 : (g > 8192 ? 8192 : g));
}

}  // namespace

int contract_plan(const char *expr, int ra, const i64 *la, const i64 *sa, int rb, const i64 *lb, const i64 *sb, int rc,
                  const i64 *lc, const i64 *sc, ddla_contract_desc *d) {
    std::string parts[3];
    int which = 0;
    for (const char *p = expr; *p; p++) {
        if (*p == ' ') continue;
        if (*p == ',') {
            if (which != 0) return -1;
            which = 1;
            continue;
        }
        if (*p == '-' && p[1] == '>') {
            if (which != 1) return -1;
            which = 2;
            p++;
            continue;
        }
        parts[which].push_back(*p);
    }
    if (which != 2) return -1;
    std::vector<Ent> A, B, C;
    if (diagonal(parts[0], ra, la, sa, A) || diagonal(parts[1], rb, lb, sb, B) || diagonal(parts[2], rc, lc, sc, C))
        return -2;
    for (auto &e : A) e.used = e.len <= 1;
    for (auto &e : B) e.used = e.len <= 1;
    for (auto &e : C) e.used = e.len <= 1;
    std::vector<ddla_contract_mode> abc, conly, aonly, bonly, M, N, K;
    for (auto &c : C) {
        if (c.used) continue;
        Ent *fa = nullptr, *fb = nullptr;
        for (auto &e : A)
            if (!e.used && e.sym == c.sym) fa = &e;
        for (auto &e : B)
            if (!e.used && e.sym == c.sym) fb = &e;
        if ((fa && fa->len != c.len) || (fb && fb->len != c.len)) return -2;
        ddla_contract_mode m{c.len, fa ? fa->stride : 0, fb ? fb->stride : 0, c.stride};
        if (fa && fb) abc.push_back(m);
        else if (fa) M.push_back(m);
        else if (fb) N.push_back(m);
        else conly.push_back(m);
        if (fa) fa->used = true;
        if (fb) fb->used = true;
        c.used = true;
    }
    for (auto &a : A) {
        if (a.used) continue;
        Ent *fb = nullptr;
        for (auto &e : B)
            if (!e.used && e.sym == a.sym) fb = &e;
        if (fb) {
            if (fb->len != a.len) return -2;
            K.push_back(ddla_contract_mode{a.len, a.stride, fb->stride, 0});
            fb->used = true;
        } else {
            aonly.push_back(ddla_contract_mode{a.len, a.stride, 0, 0});
        }
        a.used = true;
    }
    for (auto &b : B)
        if (!b.used) bonly.push_back(ddla_contract_mode{b.len, 0, b.stride, 0});
    sort_desc(abc, 2);
    sort_desc(conly, 2);
    sort_desc(aonly, 0);
    sort_desc(bonly, 1);
    std::vector<ddla_contract_mode> batch;
    for (auto *v : {&abc, &conly, &aonly, &bonly}) batch.insert(batch.end(), v->begin(), v->end());
    fold2(M, 0, 2);
    sort_desc(M, 2);
    fold2(N, 1, 2);
    sort_desc(N, 2);
    fold2(K, 0, 1);
    sort_desc(K, 0);
    if (M.empty()) M.push_back({1, 1, 1, 1});
    if (N.empty()) N.push_back({1, 1, 1, 1});
    if (K.empty()) K.push_back({1, 1, 1, 1});
    if (batch.size() > 48 || M.size() > 16 || N.size() > 16 || K.size() > 16) return -3;
    memset(d, 0, sizeof(*d));
    bool swap = N.back().sc == 1;
    if (swap) {
        std::swap(M, N);
        for (auto &m : M) { m.sa = m.sb; m.sb = 0; }
        for (auto &m : N) { m.sb = m.sa; m.sa = 0; }
        for (auto &m : K) std::swap(m.sa, m.sb);
        for (auto &m : batch) std::swap(m.sa, m.sb);
    }
    d->swapped = swap;
    d->nbatch = (int)batch.size();
    d->nm = (int)M.size();
    d->nn = (int)N.size();
    d->nk = (int)K.size();
    std::copy(batch.begin(), batch.end(), d->batch);
    std::copy(M.begin(), M.end(), d->m);
    std::copy(N.begin(), N.end(), d->n);
    std::copy(K.begin(), K.end(), d->k);
    return 0;
}

// C += alpha * A (x) B on device data according to a plan.
int contract_exec(ddla_handle h, const ddla_contract_desc *d, double alpha, const double *a, const double *b,
                  double *c, int prec) {
    if (alpha == 0.0) return 0;
    if (d->swapped) std::swap(a, b);
    cudaStream_t s = h->stream;
    const i64 M = total(d->m, d->nm), N = total(d->n, d->nn), K = total(d->k, d->nk);
    if (M == 0 || N == 0) return 0;
    // batch modes: those with a C stride (distinct outputs) go into one launch;
    // those without (summed) are looped on the host.
    std::vector<ddla_contract_mode> par, seq;
    for (int i = 0; i < d->nbatch; i++) (d->batch[i].sc != 0 ? par : seq).push_back(d->batch[i]);
    const i64 npar = total(par.data(), (int)par.size()), nseq = total(seq.data(), (int)seq.size());
    if (K == 0) return 0;
    std::vector<i64> poa = offsets(par.data(), (int)par.size(), 0), pob = offsets(par.data(), (int)par.size(), 1),
                     poc = offsets(par.data(), (int)par.size(), 2);
    std::vector<i64> soa = offsets(seq.data(), (int)seq.size(), 0), sob = offsets(seq.data(), (int)seq.size(), 1),
                     soc = offsets(seq.data(), (int)seq.size(), 2);
    const bool direct = d->nm == 1 && d->nn == 1 && d->nk == 1;
    Timed t(s, TC_CONTRACT, 2.0 * M * N * K * npar * nseq, 8.0 * (M * K + K * N + 2 * M * N) * npar * nseq);
    if (direct) {
        // offset table [npar][3] on the device
        std::vector<i64> tab((size_t)npar * 3);
        for (i64 i = 0; i < npar; i++) {
            tab[i * 3] = poa[i];
            tab[i * 3 + 1] = pob[i];
            tab[i * 3 + 2] = poc[i];
        }
        i64 *dtab;
        DDLA_TRY(workspace(h, WS_MISC, sizeof(i64) * tab.size(), (void **)&dtab));
        DDLA_CUDA(cudaMemcpyAsync(dtab, tab.data(), sizeof(i64) * tab.size(), cudaMemcpyHostToDevice, s));
        for (i64 q = 0; q < nseq; q++) {
            View<const double> Av{a + soa[q], M, K, d->m[0].sa, d->k[0].sa};
            View<const double> Bv{b + sob[q], K, N, d->k[0].sb, d->n[0].sb};
            View<double> Cv{c + soc[q], M, N, d->m[0].sc, d->n[0].sc};
            if (prec == DDLA_PREC_FP64) {
                DDLA_TRY(gemm_f64_offsets(s, M, N, K, alpha, Av, Bv, 1.0, Cv, npar, dtab));
            } else {
                DDLA_TRY(gemm_ozaki(h, M, N, K, alpha, Av, Bv, 1.0, Cv, DDLA_DENSE, npar, dtab));
            }
        }
        DDLA_CUDA(cudaStreamSynchronize(s));   // the host offset vectors go out of scope
        return 0;
    }
    // general path: gather -> dense GEMM -> scatter-add, one batch index at a time
    std::vector<i64> rA = offsets(d->m, d->nm, 0), rC = offsets(d->m, d->nm, 2), cB = offsets(d->n, d->nn, 1),
                     cC = offsets(d->n, d->nn, 2), kA = offsets(d->k, d->nk, 0), kB = offsets(d->k, d->nk, 1);
    i64 *tabs;
    const size_t ntab = rA.size() * 2 + cB.size() * 2 + kA.size() * 2;
    DDLA_TRY(workspace(h, WS_MISC, sizeof(i64) * ntab, (void **)&tabs));
    i64 *drA = tabs, *drC = drA + rA.size(), *dcB = drC + rC.size(), *dcC = dcB + cB.size(), *dkA = dcC + cC.size(),
        *dkB = dkA + kA.size();
    DDLA_CUDA(cudaMemcpyAsync(drA, rA.data(), 8 * rA.size(), cudaMemcpyHostToDevice, s));
    DDLA_CUDA(cudaMemcpyAsync(drC, rC.data(), 8 * rC.size(), cudaMemcpyHostToDevice, s));
    DDLA_CUDA(cudaMemcpyAsync(dcB, cB.data(), 8 * cB.size(), cudaMemcpyHostToDevice, s));
    DDLA_CUDA(cudaMemcpyAsync(dcC, cC.data(), 8 * cC.size(), cudaMemcpyHostToDevice, s));
    DDLA_CUDA(cudaMemcpyAsync(dkA, kA.data(), 8 * kA.size(), cudaMemcpyHostToDevice, s));
    DDLA_CUDA(cudaMemcpyAsync(dkB, kB.data(), 8 * kB.size(), cudaMemcpyHostToDevice, s));
    double *dA, *dB, *dC;
    DDLA_TRY(workspace(h, WS_A, 8 * (size_t)(M * K), (void **)&dA));
    DDLA_TRY(workspace(h, WS_B, 8 * (size_t)(K * N), (void **)&dB));
    DDLA_TRY(workspace(h, WS_C, 8 * (size_t)(M * N), (void **)&dC));
    for (i64 q = 0; q < nseq; q++)
        for (i64 p = 0; p < npar; p++) {
            k_gather<<<grid_of(M * K), 256, 0, s>>>(a + soa[q] + poa[p], drA, dkA, M, K, dA);
            DDLA_LAUNCHED();
            k_gather<<<grid_of(K * N), 256, 0, s>>>(b + sob[q] + pob[p], dkB, dcB, K, N, dB);
            DDLA_LAUNCHED();
            View<const double> Av{dA, M, K, K, 1}, Bv{dB, K, N, N, 1};
            View<double> Cv{dC, M, N, N, 1};
            if (prec == DDLA_PREC_FP64) DDLA_TRY(gemm_f64(s, M, N, K, alpha, Av, Bv, 0.0, Cv));
            else DDLA_TRY(gemm_ozaki(h, M, N, K, alpha, Av, Bv, 0.0, Cv));
            k_scatter_add<<<grid_of(M * N), 256, 0, s>>>(dC, drC, dcC, M, N, c + soc[q] + poc[p]);
            DDLA_LAUNCHED();
        }
    DDLA_CUDA(cudaStreamSynchronize(s));
    return 0;
}

}  // namespace ddla

using namespace ddla;

extern "C" {

int ddla_contract_plan(const char *expr, int32_t rank_a, const int64_t *len_a, const int64_t *str_a, int32_t rank_b,
                       const int64_t *len_b, const int64_t *str_b, int32_t rank_c, const int64_t *len_c,
                       const int64_t *str_c, ddla_contract_desc *out) {
    if (!expr) return -1;
    if (!out) return -11;
    int rc = contract_plan(expr, rank_a, len_a, str_a, rank_b, len_b, str_b, rank_c, len_c, str_c, out);
    if (rc == -1) { set_error("einsum expression must be 'A,B->C'"); return -1; }
    if (rc == -2) { set_error("einsum symbols and tensor ranks / lengths do not match"); return -2; }
    if (rc == -3) { set_error("einsum with too many modes"); return DDLA_ERR_UNSUPPORTED; }
    return 0;
}

int ddla_dev_contract(ddla_handle h, const ddla_contract_desc *d, double alpha, const double *a, const double *b,
                      double *c, int32_t precision) {
    if (!h) return -1;
    if (!d) return -2;
    if (precision != DDLA_PREC_FP64 && precision != DDLA_PREC_OZAKI) return -7;
    return contract_exec(h, d, alpha, a, b, c, precision);
}

int ddla_contract(const ddla_contract_desc *d, double alpha, const double *a, int64_t na, const double *b,
                  int64_t nb, double *c, int64_t nc, int32_t precision) {
    if (!d) return -1;
    if (na < 0) return -4;
    if (nb < 0) return -6;
    if (nc < 0) return -8;
    if (precision != DDLA_PREC_FP64 && precision != DDLA_PREC_OZAKI) return -9;
    ddla_handle h;
    DDLA_TRY(default_handle(&h));
    cudaStream_t s = h->stream;
    double *dA, *dB, *dC;
    DDLA_CUDA(cudaMallocAsync(&dA, 8 * (size_t)(na > 0 ? na : 1), s));
    DDLA_CUDA(cudaMallocAsync(&dB, 8 * (size_t)(nb > 0 ? nb : 1), s));
    DDLA_CUDA(cudaMallocAsync(&dC, 8 * (size_t)(nc > 0 ? nc : 1), s));
    DDLA_CUDA(cudaMemcpyAsync(dA, a, 8 * (size_t)na, cudaMemcpyHostToDevice, s));
    DDLA_CUDA(cudaMemcpyAsync(dB, b, 8 * (size_t)nb, cudaMemcpyHostToDevice, s));
    DDLA_CUDA(cudaMemcpyAsync(dC, c, 8 * (size_t)nc, cudaMemcpyHostToDevice, s));
    int rc = contract_exec(h, d, alpha, dA, dB, dC, precision);
    if (rc == 0) {
        DDLA_CUDA(cudaMemcpyAsync(c, dC, 8 * (size_t)nc, cudaMemcpyDeviceToHost, s));
        DDLA_CUDA(cudaStreamSynchronize(s));
    }
    cudaFreeAsync(dA, s);
    cudaFreeAsync(dB, s);
    cudaFreeAsync(dC, s);
    cudaStreamSynchronize(s);
    return rc;
}

}  // extern "C"
