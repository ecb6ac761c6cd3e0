// Multi-operand einsum: MArray.Einsum (DDLA/Einsum/MArray.Contract.cs:409-427).
//
// DDLA builds a tree of pairwise contractions greedily
// (DDLA/Einsum/EinsumTree/EinsumState.cs:45-419): at every step, over all
// pairs (l < r) of the current tensors, the pair whose result is smallest
// relative to its operands wins (cost = |result| - (|l| + |r|), ties to the
// smaller l, then the smaller r); the result keeps the symbols of l and r that
// another tensor or the target still uses, in order of first appearance, and
// takes l's place.  The last contraction writes the target directly.  Here the
// same path runs as a chain of pairwise device contractions (contract.cu) whose
// intermediates stay in device memory (stream-ordered allocations freed as soon
// as they are consumed), so a chain makes no host round trips.
#include <cstring>
#include <string>
#include <vector>

#include "common.cuh"

namespace ddla {

int contract_plan(const char *expr, int ra, const i64 *la, const i64 *sa, int rb, const i64 *lb, const i64 *sb, int rc,
                  const i64 *lc, const i64 *sc, ddla_contract_desc *d);
int contract_exec(ddla_handle h, const ddla_contract_desc *d, double alpha, const double *a, const double *b,
                  double *c, int prec);

namespace {

struct EinsumStep {
    int left, right;
    std::string a, b, out;
};

struct EinsumPath {
    std::string target;
    std::vector<std::string> inputs;
    std::vector<char> symbols;      // order of first appearance over the inputs
    std::vector<i64> len;           // per symbol
    std::vector<EinsumStep> steps;
};

int sym_index(const EinsumPath &p, char c) {
    for (size_t i = 0; i < p.symbols.size(); i++)
        if (p.symbols[i] == c) return (int)i;
    return -1;
}

// EinsumState(expression, tensors) and Parse(), EinsumState.cs:45-160, 330-408.
int einsum_path(const char *expr, int n, const int *ranks, const i64 *const *lens, EinsumPath &p) {
    std::string lhs, rhs;
    const char *arrow = strstr(expr, "->");
    if (!arrow) {
        set_error("einsum: expression needs '->'");
        return -1;
    }
    for (const char *q = expr; q < arrow; q++)
        if (*q != ' ') lhs.push_back(*q);
    for (const char *q = arrow + 2; *q; q++)
        if (*q != ' ') rhs.push_back(*q);
    p.target = rhs;
    p.inputs.clear();
    std::string cur;
    for (char c : lhs) {
        if (c == ',') {
            p.inputs.push_back(cur);
            cur.clear();
        } else {
            cur.push_back(c);
        }
    }
    p.inputs.push_back(cur);
    if ((int)p.inputs.size() != n) {
        set_error("einsum: number of tensors does not match the expression");
        return -2;
    }
    p.symbols.clear();
    p.len.clear();
    for (int i = 0; i < n; i++) {
        const std::string &nm = p.inputs[i];
        if ((int)nm.size() != ranks[i]) {
            set_error("einsum: tensor rank does not match its symbols");
            return -3;
        }
        for (int d = 0; d < ranks[i]; d++) {
            int s = sym_index(p, nm[d]);
            if (s < 0) {
                p.symbols.push_back(nm[d]);
                p.len.push_back(lens[i][d]);
            } else if (p.len[s] != lens[i][d]) {
                set_error("einsum: conflicting lengths for one symbol");
                return -4;
            }
        }
    }
    const int D = (int)p.symbols.size();
    std::vector<char> in_target(D, 0);
    for (char c : p.target) {
        int s = sym_index(p, c);
        if (s < 0 || in_target[s]) {
            set_error("einsum: target symbol missing from the inputs or repeated");
            return -5;
        }
        in_target[s] = 1;
    }
    // rows: current tensors, then the target
    std::vector<std::vector<char>> used(n, std::vector<char>(D, 0));
    for (int i = 0; i < n; i++)
        for (char c : p.inputs[i]) used[i][sym_index(p, c)] = 1;
    std::vector<std::string> names = p.inputs;
    // DDLA sizes the inputs with a product that starts from 0
    // (EinsumState.cs:122-131), so they count as 0 and only intermediates
    // count with their true size; kept, because the path fixes the order of
    // the pairwise products.
    std::vector<double> size(n, 0.0);
    p.steps.clear();
    while ((int)names.size() > 1) {
        const int cnt = (int)names.size();
        int bl = -1, br = -1;
        double bc = 0.0, brs = 0.0;
        std::string bname;
        std::vector<char> bused;
        for (int l = 0; l < cnt - 1; l++)
            for (int r = l + 1; r < cnt; r++) {
                // TryContract, EinsumState.cs:290-328
                double rs = 1.0;
                std::string name;
                std::vector<char> u(D, 0);
                for (int d = 0; d < D; d++) {
                    if (!used[l][d] && !used[r][d]) continue;
                    bool other = in_target[d] != 0;
                    for (int j = 0; j < cnt && !other; j++)
                        if (j != l && j != r && used[j][d]) other = true;
                    if (other) {
                        u[d] = 1;
                        rs *= (double)p.len[d];
                        name.push_back(p.symbols[d]);
                    }
                }
                const double cost = rs - (size[l] + size[r]);
                if (bl < 0 || cost < bc) {
                    bl = l;
                    br = r;
                    bc = cost;
                    brs = rs;
                    bname = name;
                    bused = u;
                }
            }
        p.steps.push_back(EinsumStep{bl, br, names[bl], names[br], bname});
        names[bl] = bname;
        size[bl] = brs;
        used[bl] = bused;
        names.erase(names.begin() + br);
        size.erase(size.begin() + br);
        used.erase(used.begin() + br);
    }
    // OutputNode renames the last contraction to the target (EinsumNodes.cs:82-93)
    if (!p.steps.empty()) p.steps.back().out = p.target;
    return 0;
}

// A tensor of the chain: an input (caller's strides) or an intermediate
// (row-major over its symbols).
struct Slot {
    std::string name;
    const double *p;
    double *owned;
    std::vector<i64> len, str;
};

struct NdArgs {
    int rank;
    i64 len[16], str[16];
};

// x = beta * x over a strided tensor (beta == 0 writes zeros).
__global__ void k_scale_nd(NdArgs a, double beta, double *x, i64 total) {
    for (i64 e = blockIdx.x * (i64)blockDim.x + threadIdx.x; e < total; e += (i64)gridDim.x * blockDim.x) {
        i64 rem = e, off = 0;
        for (int d = a.rank - 1; d >= 0; d--) {
            off += (rem % a.len[d]) * a.str[d];
            rem /= a.len[d];
        }
        x[off] = beta == 0.0 ? 0.0 : beta * x[off];
    }
}

const double k_one = 1.0;

}  // namespace

int einsum_exec(ddla_handle h, const char *expr, int n, const int *ranks, const i64 *const *lens,
                const i64 *const *strides, const double *const *inputs, double alpha, double beta, int rank_out,
                const i64 *len_out, const i64 *str_out, double *out, int prec) {
    EinsumPath p;
    DDLA_TRY(einsum_path(expr, n, ranks, lens, p));
    if ((int)p.target.size() != rank_out) {
        set_error("einsum: output rank does not match the target");
        return -10;
    }
    for (int d = 0; d < rank_out; d++)
        if (len_out[d] != p.len[sym_index(p, p.target[d])]) {
            set_error("einsum: output lengths do not match the target");
            return -11;
        }
    if (rank_out > 16) {
        set_error("einsum: output rank above 16");
        return DDLA_ERR_UNSUPPORTED;
    }
    cudaStream_t s = h->stream;
    i64 total = 1;
    for (int d = 0; d < rank_out; d++) total *= len_out[d];
    if (beta != 1.0 && total > 0) {
        NdArgs a{};
        a.rank = rank_out;
        for (int d = 0; d < rank_out; d++) {
            a.len[d] = len_out[d];
            a.str[d] = str_out[d];
        }
        const i64 blocks = (total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096;
        k_scale_nd<<<(unsigned)blocks, 256, 0, s>>>(a, beta, out, total);
        DDLA_LAUNCHED();
    }
    if (total == 0 || alpha == 0.0) return 0;
    std::vector<Slot> slots(n);
    for (int i = 0; i < n; i++) {
        slots[i].name = p.inputs[i];
        slots[i].p = inputs[i];
        slots[i].owned = nullptr;
        slots[i].len.assign(lens[i], lens[i] + ranks[i]);
        slots[i].str.assign(strides[i], strides[i] + ranks[i]);
    }
    // a single operand: contracted with the scalar 1 ("ij,->ji"), which covers
    // transposes, diagonals and sums
    if (p.steps.empty()) {
        Slot one{"", &k_one, nullptr, {}, {}};
        double *d_one;
        DDLA_CUDA(cudaMallocAsync(&d_one, sizeof(double), s));
        DDLA_CUDA(cudaMemcpyAsync(d_one, &k_one, sizeof(double), cudaMemcpyHostToDevice, s));
        one.p = d_one;
        one.owned = d_one;
        slots.push_back(one);
        p.steps.push_back(EinsumStep{0, 1, p.inputs[0], "", p.target});
    }
    int rc = 0;
    for (size_t si = 0; si < p.steps.size() && rc == 0; si++) {
        const EinsumStep &st = p.steps[si];
        const bool last = si + 1 == p.steps.size();
        Slot &A = slots[st.left], &B = slots[st.right];
        Slot R;
        R.name = st.out;
        R.owned = nullptr;
        if (last) {
            R.len.assign(len_out, len_out + rank_out);
            R.str.assign(str_out, str_out + rank_out);
            R.p = out;
        } else {
            i64 cnt = 1;
            for (char c : st.out) R.len.push_back(p.len[sym_index(p, c)]);
            R.str.assign(R.len.size(), 1);
            for (int d = (int)R.len.size() - 1; d >= 0; d--) {
                R.str[d] = cnt;
                cnt *= R.len[d];
            }
            rc = cudaMallocAsync(&R.owned, sizeof(double) * (size_t)(cnt > 0 ? cnt : 1), s) == cudaSuccess
                     ? 0
                     : DDLA_ERR_NOMEM;
            if (rc) break;
            cudaMemsetAsync(R.owned, 0, sizeof(double) * (size_t)cnt, s);
            R.p = R.owned;
        }
        const std::string e = st.a + "," + st.b + "->" + st.out;
        ddla_contract_desc d;
        rc = contract_plan(e.c_str(), (int)A.len.size(), A.len.data(), A.str.data(), (int)B.len.size(), B.len.data(),
                           B.str.data(), (int)R.len.size(), R.len.data(), R.str.data(), &d);
        if (rc) {
            set_error("einsum: a pairwise step could not be planned");
            rc = DDLA_ERR_UNSUPPORTED;
            break;
        }
        rc = contract_exec(h, &d, last ? alpha : 1.0, A.p, B.p, (double *)R.p, prec);
        if (A.owned) cudaFreeAsync(A.owned, s);
        if (B.owned) cudaFreeAsync(B.owned, s);
        A.owned = B.owned = nullptr;
        slots[st.left] = R;
        slots.erase(slots.begin() + st.right);
    }
    for (auto &sl : slots)
        if (sl.owned && sl.p != out) cudaFreeAsync(sl.owned, s);
    return rc;
}

int einsum_path_string(const char *expr, int n, const int *ranks, const i64 *const *lens, std::string &outs) {
    EinsumPath p;
    DDLA_TRY(einsum_path(expr, n, ranks, lens, p));
    outs.clear();
    for (size_t i = 0; i < p.steps.size(); i++) {
        if (i) outs.push_back(';');
        outs += p.steps[i].a + "," + p.steps[i].b + "->" + p.steps[i].out;
    }
    return 0;
}

}  // namespace ddla

using namespace ddla;

extern "C" {

int ddla_einsum_path(const char *expr, int32_t n_inputs, const int32_t *ranks, const int64_t *const *lens, char *buf,
                     int32_t buflen) {
    if (!expr) return -1;
    if (n_inputs < 1) return -2;
    if (!ranks) return -3;
    if (!lens) return -4;
    if (!buf || buflen < 1) return -5;
    std::string s;
    DDLA_TRY(einsum_path_string(expr, n_inputs, ranks, lens, s));
    if ((int)s.size() + 1 > buflen) {
        set_error("einsum_path: buffer too small");
        return -6;
    }
    memcpy(buf, s.c_str(), s.size() + 1);
    return 0;
}

int ddla_dev_einsum(ddla_handle h, const char *expr, int32_t n_inputs, const int32_t *ranks,
                    const int64_t *const *lens, const int64_t *const *strides, const double *const *inputs,
                    double alpha, double beta, int32_t rank_out, const int64_t *len_out, const int64_t *str_out,
                    double *out, int32_t precision) {
    if (!h) return -1;
    if (!expr) return -2;
    if (n_inputs < 1) return -3;
    if (!ranks || !lens || !strides || !inputs) return -4;
    if (rank_out < 0 || (rank_out > 0 && (!len_out || !str_out))) return -10;
    if (precision != DDLA_PREC_FP64 && precision != DDLA_PREC_OZAKI) return -14;
    return einsum_exec(h, expr, n_inputs, ranks, lens, strides, inputs, alpha, beta, rank_out, len_out, str_out, out,
                       precision);
}

int ddla_einsum(const char *expr, int32_t n_inputs, const int32_t *ranks, const int64_t *const *lens,
                const int64_t *const *strides, const double *const *inputs, const int64_t *counts, double alpha,
                double beta, int32_t rank_out, const int64_t *len_out, const int64_t *str_out, double *out,
                int64_t out_count, int32_t precision) {
    if (!expr) return -1;
    if (n_inputs < 1) return -2;
    if (!ranks || !lens || !strides || !inputs || !counts) return -3;
    if (rank_out < 0 || (rank_out > 0 && (!len_out || !str_out))) return -10;
    if (out_count < 0) return -14;
    if (precision != DDLA_PREC_FP64 && precision != DDLA_PREC_OZAKI) return -15;
    ddla_handle h;
    DDLA_TRY(default_handle(&h));
    cudaStream_t s = h->stream;
    std::vector<double *> din(n_inputs, nullptr);
    double *dout = nullptr;
    int rc = 0;
    for (int i = 0; i < n_inputs && rc == 0; i++) {
        const size_t bytes = 8 * (size_t)(counts[i] > 0 ? counts[i] : 1);
        if (cudaMallocAsync(&din[i], bytes, s) != cudaSuccess) rc = DDLA_ERR_NOMEM;
        else if (counts[i] > 0 &&
                 cudaMemcpyAsync(din[i], inputs[i], 8 * (size_t)counts[i], cudaMemcpyHostToDevice, s) != cudaSuccess)
            rc = DDLA_ERR_CUDA;
    }
    if (rc == 0 && cudaMallocAsync(&dout, 8 * (size_t)(out_count > 0 ? out_count : 1), s) != cudaSuccess)
        rc = DDLA_ERR_NOMEM;
    if (rc == 0 && out_count > 0 && beta != 0.0 &&
        cudaMemcpyAsync(dout, out, 8 * (size_t)out_count, cudaMemcpyHostToDevice, s) != cudaSuccess)
        rc = DDLA_ERR_CUDA;
    if (rc == 0) {
        std::vector<const double *> cin(din.begin(), din.end());
        rc = einsum_exec(h, expr, n_inputs, ranks, lens, strides, cin.data(), alpha, beta, rank_out, len_out, str_out,
                         dout, precision);
    }
    if (rc == 0 && out_count > 0) {
        // copy back only the elements of the output view
        std::vector<double> tmp((size_t)out_count);
        if (cudaMemcpyAsync(tmp.data(), dout, 8 * (size_t)out_count, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            rc = DDLA_ERR_CUDA;
        } else {
            i64 total = 1;
            for (int d = 0; d < rank_out; d++) total *= len_out[d];
            for (i64 e = 0; e < total; e++) {
                i64 rem = e, off = 0;
                for (int d = rank_out - 1; d >= 0; d--) {
                    off += (rem % len_out[d]) * str_out[d];
                    rem /= len_out[d];
                }
                out[off] = tmp[(size_t)off];
            }
        }
    }
    for (auto *pp : din)
        if (pp) cudaFreeAsync(pp, s);
    if (dout) cudaFreeAsync(dout, s);
    cudaStreamSynchronize(s);
    return rc;
}

}  // extern "C"
