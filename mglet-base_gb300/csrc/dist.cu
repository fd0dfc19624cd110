// dist.cu -- grid-partitioned runs: halo-grid refresh and cross-rank
// reductions (plain form, one level).
//
// The reference's connect sends the boxes a remote grid needs and receives
// its own ghost boxes (connect2_mod.F90:406-548, recv_all / send_all /
// process_bufs); its pressure solve all-reduces the maximum residual
// (pressuresolver_mod.F90:295).  Here a rank keeps read-only copies of the
// remote grids next to its own ("halo grids"); the boxes of those copies that
// its connects read are refreshed from their owners at the start of every
// connect, after which the ordinary single-rank task list runs unchanged.
// The exchange itself is the caller's: the library packs its owned boxes per
// peer (one kernel per field), copies them to pinned host buffers, calls the
// exchange function, and unpacks what came back into the copies.
#include <algorithm>
#include <cstring>
#include <map>
#include <vector>

#include "internal.h"

namespace mg {

struct PartBox {
    long long off;      // element offset of the box origin in the field
    int nk, nj, ni;
    int kk, kj;         // grid strides
    long long pbase;    // points of the peers before this box's peer
    long long ppts;     // points of this box's peer (one field)
    long long boff;     // offset of the box inside its peer's field block
};

struct Part {
    mglet_exchange_fn fn = nullptr;
    void* user = nullptr;
    std::vector<int> peers;                     // sorted
    std::vector<long long> sendpts, recvpts;    // per peer, one field
    long long sendtot = 0, recvtot = 0;
    PartBox *d_send = nullptr, *d_recv = nullptr;
    int nsend = 0, nrecv = 0;
    double *d_sbuf = nullptr, *d_rbuf = nullptr;   // [6 * tot]
    double *h_sbuf = nullptr, *h_rbuf = nullptr;   // pinned
};

namespace {

// box b of the table into (or out of) the buffer block of field s of nf
__global__ void k_part_pack(const PartBox* __restrict__ boxes, const double* __restrict__ f,
                            double* __restrict__ buf, int s, int nf) {
    const PartBox B = boxes[blockIdx.x];
    const int n = B.nk * B.nj * B.ni;
    double* dst = buf + nf * B.pbase + s * B.ppts + B.boff;
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const int k = t % B.nk, j = (t / B.nk) % B.nj, i = t / (B.nk * B.nj);
        dst[t] = f[B.off + (long long)i * B.kj + (long long)j * B.kk + k];
    }
}

__global__ void k_part_unpack(const PartBox* __restrict__ boxes, double* __restrict__ f,
                              const double* __restrict__ buf, int s, int nf) {
    const PartBox B = boxes[blockIdx.x];
    const int n = B.nk * B.nj * B.ni;
    const double* src = buf + nf * B.pbase + s * B.ppts + B.boff;
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const int k = t % B.nk, j = (t / B.nk) % B.nj, i = t / (B.nk * B.nj);
        f[B.off + (long long)i * B.kj + (long long)j * B.kk + k] = src[t];
    }
}

int build_boxes(Ctx* c, const int32_t* rows, int n, const std::vector<int>& peers,
                std::vector<long long>& pts, std::vector<PartBox>& out) {
    pts.assign(peers.size(), 0);
    out.clear();
    for (int r = 0; r < n; ++r) {
        const int32_t* w = rows + 8 * r;
        const int q = (int)(std::lower_bound(peers.begin(), peers.end(), w[0]) - peers.begin());
        const int g = w[1];
        if (g < 1 || g > c->ngrid) {
            set_error("set_partition: grid out of range");
            return MGLET_ERR_ARG;
        }
        const DevGrid& G = c->grids[g - 1];
        const int k0 = w[2], k1 = w[3], j0 = w[4], j1 = w[5], i0 = w[6], i1 = w[7];
        if (k0 < 1 || k1 > G.kk || k0 > k1 || j0 < 1 || j1 > G.jj || j0 > j1 || i0 < 1 ||
            i1 > G.ii || i0 > i1) {
            set_error("set_partition: box outside its grid");
            return MGLET_ERR_ARG;
        }
        PartBox b;
        b.off = G.ip3 + (long long)(i0 - 1) * G.kk * G.jj + (long long)(j0 - 1) * G.kk + (k0 - 1);
        b.nk = k1 - k0 + 1; b.nj = j1 - j0 + 1; b.ni = i1 - i0 + 1;
        b.kk = G.kk; b.kj = G.kk * G.jj;
        b.pbase = q;          // peer index for now
        b.boff = pts[q];
        pts[q] += (long long)b.nk * b.nj * b.ni;
        out.push_back(b);
    }
    std::vector<long long> base(peers.size() + 1, 0);
    for (size_t q = 0; q < peers.size(); ++q) base[q + 1] = base[q] + pts[q];
    for (PartBox& b : out) {
        const int q = (int)b.pbase;
        b.pbase = base[q];
        b.ppts = pts[q];
    }
    return 0;
}

}  // namespace

void part_release(Ctx* c) {
    Part* p = c->part;
    if (!p) return;
    for (void* a : {(void*)p->d_send, (void*)p->d_recv, (void*)p->d_sbuf, (void*)p->d_rbuf})
        cudaFree(a);
    if (p->h_sbuf) cudaFreeHost(p->h_sbuf);
    if (p->h_rbuf) cudaFreeHost(p->h_rbuf);
    delete p;
    c->part = nullptr;
}

int set_partition(Ctx* c, const int32_t* halo, int nsend, const int32_t* send, int nrecv,
                  const int32_t* recv, mglet_exchange_fn fn, void* user) {
    if (c->prm.form != MGLET_FORM_PLAIN || c->minlevel != c->maxlevel) {
        set_error("set_partition: the plain form on one grid level only");
        return MGLET_ERR_UNSUPPORTED;
    }
    if (!halo || !fn || nsend < 0 || nrecv < 0 || (nsend && !send) || (nrecv && !recv)) {
        set_error("set_partition: bad arguments");
        return MGLET_ERR_ARG;
    }
    part_release(c);
    Part* p = new Part();
    c->part = p;
    p->fn = fn;
    p->user = user;
    for (int g = 0; g < c->ngrid; ++g) c->grids[g].halo = halo[g] != 0;
    MG_CUDA(copy_on(c->stream, c->d_grids, c->grids.data(), c->ngrid * sizeof(DevGrid),
                    cudaMemcpyHostToDevice));
    for (int r = 0; r < nsend; ++r) p->peers.push_back(send[8 * r]);
    for (int r = 0; r < nrecv; ++r) p->peers.push_back(recv[8 * r]);
    std::sort(p->peers.begin(), p->peers.end());
    p->peers.erase(std::unique(p->peers.begin(), p->peers.end()), p->peers.end());
    std::vector<PartBox> sb, rb;
    if (int rc = build_boxes(c, send, nsend, p->peers, p->sendpts, sb)) return rc;
    if (int rc = build_boxes(c, recv, nrecv, p->peers, p->recvpts, rb)) return rc;
    for (long long v : p->sendpts) p->sendtot += v;
    for (long long v : p->recvpts) p->recvtot += v;
    p->nsend = (int)sb.size();
    p->nrecv = (int)rb.size();
    auto up = [&](const std::vector<PartBox>& v, PartBox** d) -> int {
        if (v.empty()) return 0;
        MG_CUDA(cudaMalloc(d, v.size() * sizeof(PartBox)));
        MG_CUDA(copy_on(c->stream, *d, v.data(), v.size() * sizeof(PartBox), cudaMemcpyHostToDevice));
        return 0;
    };
    if (int rc = up(sb, &p->d_send)) return rc;
    if (int rc = up(rb, &p->d_recv)) return rc;
    const size_t ns = (size_t)std::max(1LL, 6 * p->sendtot), nr = (size_t)std::max(1LL, 6 * p->recvtot);
    MG_CUDA(cudaMalloc(&p->d_sbuf, ns * sizeof(double)));
    MG_CUDA(cudaMalloc(&p->d_rbuf, nr * sizeof(double)));
    MG_CUDA(cudaMallocHost(&p->h_sbuf, ns * sizeof(double)));
    MG_CUDA(cudaMallocHost(&p->h_rbuf, nr * sizeof(double)));
    return 0;
}

// Refreshes the halo copies of the present fields (the slots of one connect).
int part_exchange(Ctx* c, double* const fields[6]) {
    Part* p = c->part;
    if (!p) return 0;
    int nf = 0;
    for (int q = 0; q < 6; ++q) nf += fields[q] != nullptr;
    int s = 0;
    for (int q = 0; q < 6; ++q) {
        if (!fields[q]) continue;
        if (p->nsend) {
            k_part_pack<<<p->nsend, 128, 0, c->stream>>>(p->d_send, fields[q], p->d_sbuf, s, nf);
            MG_LAUNCHED(c);
        }
        ++s;
    }
    if (p->sendtot)
        MG_CUDA(cudaMemcpyAsync(p->h_sbuf, p->d_sbuf, (size_t)nf * p->sendtot * sizeof(double),
                                cudaMemcpyDeviceToHost, c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
    const int np = (int)p->peers.size();
    std::vector<double*> sp(np), rp(np);
    std::vector<int64_t> sn(np), rn(np);
    long long so = 0, ro = 0;
    for (int q = 0; q < np; ++q) {
        sp[q] = p->h_sbuf + so;
        rp[q] = p->h_rbuf + ro;
        sn[q] = nf * p->sendpts[q];
        rn[q] = nf * p->recvpts[q];
        so += sn[q];
        ro += rn[q];
    }
    if (np && p->fn(p->user, 0, np, p->peers.data(), sp.data(), sn.data(), rp.data(), rn.data())) {
        set_error("partition: the exchange function failed");
        return MGLET_ERR_ARG;
    }
    if (p->recvtot)
        MG_CUDA(cudaMemcpyAsync(p->d_rbuf, p->h_rbuf, (size_t)nf * p->recvtot * sizeof(double),
                                cudaMemcpyHostToDevice, c->stream));
    s = 0;
    for (int q = 0; q < 6; ++q) {
        if (!fields[q]) continue;
        if (p->nrecv) {
            k_part_unpack<<<p->nrecv, 128, 0, c->stream>>>(p->d_recv, fields[q], p->d_rbuf, s, nf);
            MG_LAUNCHED(c);
        }
        ++s;
    }
    return 0;
}

// v[0..n) <- its maximum (op 1) or sum (op 2) over all ranks.
int part_allreduce(Ctx* c, double* v, int n, int op) {
    Part* p = c->part;
    if (!p) return 0;
    double* b[1] = {v};
    int64_t cnt[1] = {n};
    if (p->fn(p->user, op, 0, nullptr, b, cnt, nullptr, nullptr)) {
        set_error("partition: the reduction failed");
        return MGLET_ERR_ARG;
    }
    return 0;
}

}  // namespace mg
