// hcore-gb300 — one panel step of a tile low-rank (TLR) Cholesky factorization.
//
// HiCMA factors a TLR matrix (dense diagonal tiles, low-rank off-diagonal
// tiles A_ij = U_ij V_ij^T) with a task graph whose panel k is, in order:
//   POTRF  D_kk = L_kk L_kk^T                        (hcore_dpotrf.c:23-34)
//   TRSM   A_ik <- A_ik L_kk^-T, i.e. V_ik <- L_kk^-1 V_ik   (hcore_dtrsm.c:24-48)
//   SYRK   D_ii <- D_ii - A_ik A_ik^T, i > k          (hcore_dsyrk.c:47-189)
//   GEMM   A_ij <- A_ij - A_ik A_jk^T, k < j < i, recompressed (hcore_dgemm.c:703)
// hcore_gpu_tlr_panel_step runs the whole panel on the GPU with the
// library's batched kernels: one POTRF, one batched TRSM over the panel's V
// factors, and then the dense SYRK batch and the low-rank GEMM plan
// concurrently on two streams (they touch disjoint tiles).
#include <cuda_runtime.h>

#include <vector>

#include "hc_host.h"
#include "hcore.h"

using namespace hc;

extern "C" int hcore_gpu_tlr_panel_step(const hcore_tlr_matrix *A, int k, double acc, int maxrk,
                                        int *info, int *status, void *stream) {
    if (!A || !A->D || !A->U || !A->V || !A->rank || A->nt < 1 || A->nb < 1 || k < 0 ||
        k >= A->nt || A->ldd < A->nb || A->maxrank < 1 || maxrk < 1 || !(acc >= 0)) {
        set_error("hcore_gpu_tlr_panel_step: invalid argument");
        return HCORE_GPU_EINVAL;
    }
    const int nt = A->nt, nb = A->nb;
    auto at = [nt](int i, int j) { return (size_t)i + (size_t)j * nt; };
    for (int i = k + 1; i < nt; ++i)
        for (int j = k; j < i; ++j)
            if (A->rank[at(i, j)] < 0 || A->rank[at(i, j)] > A->maxrank ||
                (A->rank[at(i, j)] > 0 && (!A->U[at(i, j)] || !A->V[at(i, j)]))) {
                set_error("hcore_gpu_tlr_panel_step: tile (%d, %d) has rank %d (storage %d)", i,
                          j, A->rank[at(i, j)], A->maxrank);
                return HCORE_GPU_EINVAL;
            }
    if (status)
        for (int i = 0; i < nt; ++i)
            for (int j = 0; j < nt; ++j) status[at(i, j)] = HCORE_GPU_S_OK;
    cudaStream_t s = (cudaStream_t)stream;

    // POTRF of the diagonal tile (lower: L_kk overwrites its lower triangle)
    hcore_potrf_task pt{'L', nb, A->D[k], A->ldd};
    int pinfo = 0;
    int rc = hcore_gpu_potrf_batched(1, &pt, &pinfo, stream);
    if (info) *info = pinfo;
    if (rc) return rc;
    if (pinfo != 0) {
        set_error("hcore_gpu_tlr_panel_step: POTRF of tile %d failed (info %d)", k, pinfo);
        return HCORE_GPU_ETASK;
    }

    // TRSM of every panel V factor with the new L_kk (tiles of rank 0 hold
    // nothing to solve)
    std::vector<hcore_trsm_task> tr;
    for (int i = k + 1; i < nt; ++i) {
        const int r = A->rank[at(i, k)];
        if (r > 0)
            tr.push_back(hcore_trsm_task{HCORE_Left, HCORE_Lower, HCORE_NoTrans, HCORE_NonUnit, nb,
                                         r, 1.0, A->D[k], A->ldd, A->V[at(i, k)], nb});
    }
    if (!tr.empty()) {
        rc = hcore_gpu_trsm_batched((int)tr.size(), tr.data(), stream);
        if (rc) return rc;
    }

    // SYRK of the later diagonal tiles and the Schur updates of the trailing
    // low-rank tiles: independent, so the GEMM plan runs on `stream` while
    // the SYRK batch runs on a side stream
    std::vector<hcore_dense_task> sy;
    for (int i = k + 1; i < nt; ++i) {
        const int r = A->rank[at(i, k)];
        if (r == 0) continue;  // A_ik = 0: D_ii is unchanged
        hcore_dense_task t{};
        t.kind = 0;
        t.M = nb;
        t.a = r;
        t.alpha = -1.0;
        t.Au = A->U[at(i, k)];
        t.Av = A->V[at(i, k)];
        t.lda = nb;
        t.CD = A->D[i];
        t.ldcd = A->ldd;
        sy.push_back(t);
    }
    std::vector<hcore_lr_task> lr;
    std::vector<size_t> slot;
    for (int j = k + 1; j < nt; ++j)
        for (int i = j + 1; i < nt; ++i) {
            const int a = A->rank[at(i, k)], b = A->rank[at(j, k)];
            if (a == 0 || b == 0) continue;  // A_ik A_jk^T = 0: A_ij is unchanged
            hcore_lr_task t{};
            t.M = nb;
            t.a = a;
            t.b = b;
            t.c = A->rank[at(i, j)];
            t.rk = 0;
            t.maxrk = maxrk;
            t.ld_newv = 0;  // 2 maxrk, the split API's rule (hcore_dgemm.c:1480)
            t.storage_maxrank = A->maxrank;
            t.alpha = -1.0;
            t.beta = 1.0;
            t.acc = acc;
            t.AU = A->U[at(i, k)];
            t.AV = A->V[at(i, k)];
            t.lda = nb;
            t.BU = A->U[at(j, k)];
            t.BV = A->V[at(j, k)];
            t.ldb = nb;
            t.CU = A->U[at(i, j)];
            t.CV = A->V[at(i, j)];
            t.ldc = nb;
            t.CUo = A->U[at(i, j)];
            t.CVo = A->V[at(i, j)];
            t.ldco = nb;
            lr.push_back(t);
            slot.push_back(at(i, j));
        }
    hcore_gpu_plan plan = nullptr;
    if (!lr.empty()) {
        rc = hcore_gpu_plan_create(&plan, HCORE_GPU_F64, (int)lr.size(), lr.data(), 0);
        if (rc) return rc;
        rc = hcore_gpu_plan_execute(plan, stream);
        if (rc) {
            hcore_gpu_plan_destroy(plan);
            return rc;
        }
    }
    if (!sy.empty()) {
        // everything queued on `stream` before the plan has completed (the
        // POTRF and TRSM calls are synchronous), so the side stream needs no
        // ordering against it and overlaps the plan
        cudaStream_t side = nullptr;
        cudaError_t e = cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            set_error("hcore_gpu_tlr_panel_step: %s", cudaGetErrorString(e));
            rc = HCORE_GPU_ECUDA;
        } else {
            rc = hcore_gpu_dense_batched((int)sy.size(), sy.data(), side);
            cudaStreamDestroy(side);
        }
        if (rc) {
            if (plan) {
                cudaStreamSynchronize(s);
                hcore_gpu_plan_destroy(plan);
            }
            return rc;
        }
    }
    if (!plan) return HCORE_GPU_OK;
    std::vector<int> rk(lr.size()), st(lr.size());
    rc = hcore_gpu_plan_results(plan, rk.data(), st.data(), stream);
    hcore_gpu_plan_destroy(plan);
    if (rc) return rc;
    bool failed = false;
    for (size_t q = 0; q < lr.size(); ++q) {
        if (st[q] == HCORE_GPU_S_OK)
            A->rank[slot[q]] = rk[q];
        else
            failed = true;
        if (status) status[slot[q]] = st[q];
    }
    if (failed) {
        set_error("hcore_gpu_tlr_panel_step: some Schur updates of panel %d failed (see status)",
                  k);
        return HCORE_GPU_ETASK;
    }
    return HCORE_GPU_OK;
}
