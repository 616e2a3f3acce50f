// Solves and field evaluation of the device-resident solver.
//   * solve_qr: dense least squares by Householder QR in the assembly
//     precision, the sequence of the reference's qrSolver
//     (numerical.cu:599-623): geqrf, unmqr (B := Q^H B), trsm (R X = B).
//   * solve_refined: min ||A x - b|| for the CHIEF-augmented (N+M) x N system
//     through its normal equations A^H A x = A^H b.  The outer loop is FP64
//     iterative refinement (residual r = b - A x and g = A^H r with FP64
//     accumulation); each correction solves A^H A d = g with GMRES whose
//     operator products run in FP32 on the c64 matrix and whose Arnoldi
//     (classical Gram-Schmidt, twice), Givens rotations and back
//     substitution run in FP64 on the device.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "solver.h"

using namespace bem;

namespace {

void cusolver_check(cusolverStatus_t s, const char *what) {
    if (s != CUSOLVER_STATUS_SUCCESS)
        BEM_FAIL(BEM_ERR_CUDA, std::string(what) + " failed (cusolver status " + std::to_string((int)s) + ")");
}
void cublas_check(cublasStatus_t s, const char *what) {
    if (s != CUBLAS_STATUS_SUCCESS)
        BEM_FAIL(BEM_ERR_CUDA, std::string(what) + " failed (cublas status " + std::to_string((int)s) + ")");
}

}  // namespace

void bem_solver_s::solve_qr() {
    const int m = R, n = N;
    BEM_PROF(prec == BEM_PREC_C64 ? "cusolver_qr_c64" : "cusolver_qr_c128", stream);
    if (prec == BEM_PREC_C64) {
        q_A.ensure(sizeof(float2) * (size_t)m * n);
        q_B.ensure(sizeof(float2) * (size_t)m * S);
        launch_to_colmajor(BEM_PREC_C64, d_A.p, lda, m, n, BEM_PREC_C64, q_A.p, m, stream);
        launch_cast(m * S, d_B.as<double2>(), q_B.as<float2>(), stream);
        int lw1 = 0, lw2 = 0;
        cusolver_check(cusolverDnCgeqrf_bufferSize(cusolver, m, n, q_A.as<cuComplex>(), m, &lw1), "Cgeqrf_bufferSize");
        q_tau.ensure(sizeof(cuComplex) * n);
        cusolver_check(cusolverDnCunmqr_bufferSize(cusolver, CUBLAS_SIDE_LEFT, CUBLAS_OP_C, m, S, n,
                                                   q_A.as<cuComplex>(), m, q_tau.as<cuComplex>(),
                                                   q_B.as<cuComplex>(), m, &lw2), "Cunmqr_bufferSize");
        q_work.ensure(sizeof(cuComplex) * std::max(1, std::max(lw1, lw2)));
        q_info.ensure(sizeof(int));
        cusolver_check(cusolverDnCgeqrf(cusolver, m, n, q_A.as<cuComplex>(), m, q_tau.as<cuComplex>(),
                                        q_work.as<cuComplex>(), std::max(lw1, lw2), q_info.as<int>()), "Cgeqrf");
        cusolver_check(cusolverDnCunmqr(cusolver, CUBLAS_SIDE_LEFT, CUBLAS_OP_C, m, S, n, q_A.as<cuComplex>(), m,
                                        q_tau.as<cuComplex>(), q_B.as<cuComplex>(), m, q_work.as<cuComplex>(),
                                        std::max(lw1, lw2), q_info.as<int>()), "Cunmqr");
        cuComplex one = make_cuComplex(1.f, 0.f);
        cublas_check(cublasCtrsm(cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N,
                                 CUBLAS_DIAG_NON_UNIT, n, S, &one, q_A.as<cuComplex>(), m,
                                 q_B.as<cuComplex>(), m), "Ctrsm");
        for (int s = 0; s < S; s++)
            launch_cast_up(n, q_B.as<float2>() + (size_t)s * m, d_x.as<double2>() + (size_t)s * n, stream);
    } else {
        q_A.ensure(sizeof(double2) * (size_t)m * n);
        q_B.ensure(sizeof(double2) * (size_t)m * S);
        launch_to_colmajor(BEM_PREC_C128, d_A.p, lda, m, n, BEM_PREC_C128, q_A.p, m, stream);
        CUDA_TRY(cudaMemcpyAsync(q_B.p, d_B.p, sizeof(double2) * (size_t)m * S, cudaMemcpyDeviceToDevice, stream));
        int lw1 = 0, lw2 = 0;
        cusolver_check(cusolverDnZgeqrf_bufferSize(cusolver, m, n, q_A.as<cuDoubleComplex>(), m, &lw1), "Zgeqrf_bufferSize");
        q_tau.ensure(sizeof(cuDoubleComplex) * n);
        cusolver_check(cusolverDnZunmqr_bufferSize(cusolver, CUBLAS_SIDE_LEFT, CUBLAS_OP_C, m, S, n,
                                                   q_A.as<cuDoubleComplex>(), m, q_tau.as<cuDoubleComplex>(),
                                                   q_B.as<cuDoubleComplex>(), m, &lw2), "Zunmqr_bufferSize");
        q_work.ensure(sizeof(cuDoubleComplex) * std::max(1, std::max(lw1, lw2)));
        q_info.ensure(sizeof(int));
        cusolver_check(cusolverDnZgeqrf(cusolver, m, n, q_A.as<cuDoubleComplex>(), m, q_tau.as<cuDoubleComplex>(),
                                        q_work.as<cuDoubleComplex>(), std::max(lw1, lw2), q_info.as<int>()), "Zgeqrf");
        cusolver_check(cusolverDnZunmqr(cusolver, CUBLAS_SIDE_LEFT, CUBLAS_OP_C, m, S, n,
                                        q_A.as<cuDoubleComplex>(), m, q_tau.as<cuDoubleComplex>(),
                                        q_B.as<cuDoubleComplex>(), m, q_work.as<cuDoubleComplex>(),
                                        std::max(lw1, lw2), q_info.as<int>()), "Zunmqr");
        cuDoubleComplex one = make_cuDoubleComplex(1.0, 0.0);
        cublas_check(cublasZtrsm(cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N,
                                 CUBLAS_DIAG_NON_UNIT, n, S, &one, q_A.as<cuDoubleComplex>(), m,
                                 q_B.as<cuDoubleComplex>(), m), "Ztrsm");
        for (int s = 0; s < S; s++)
            CUDA_TRY(cudaMemcpyAsync(d_x.as<double2>() + (size_t)s * n, q_B.as<double2>() + (size_t)s * m,
                                     sizeof(double2) * n, cudaMemcpyDeviceToDevice, stream));
    }
    int info = 0;
    CUDA_TRY(cudaMemcpyAsync(&info, q_info.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    if (info != 0) BEM_FAIL(BEM_ERR_NUMERIC, "QR reported info = " + std::to_string(info));
}

void bem_solver_s::solve_refined(bem_solve_info_t *info) {
    BEM_HOST_PROF("solve_refined");
    const int n = N, m = std::max(1, opt.max_iter);
    const int ldh = m + 1;
    const float2 *A = d_A.as<float2>();
    w_V.ensure(sizeof(double2) * (size_t)n * (m + 1));
    w_Vff.ensure(sizeof(float4) * (size_t)n * (m + 1));
    float4 *Vff = w_Vff.as<float4>();
    w_H.ensure(sizeof(double2) * (size_t)ldh * m);
    w_cs.ensure(sizeof(double2) * m);
    w_sn.ensure(sizeof(double2) * m);
    w_g.ensure(sizeof(double2) * (m + 1));
    w_y.ensure(sizeof(double2) * m);
    w_h1.ensure(sizeof(double2) * (m + 1));
    w_h2.ensure(sizeof(double2) * (m + 1));
    w_w.ensure(sizeof(double2) * n);
    w_t.ensure(sizeof(float2) * R);
    w_r.ensure(sizeof(double2) * R);
    w_gv.ensure(sizeof(double2) * n);
    // c64 copy of v_j and the float head/tail split of x (residual; the tail
    // at an even offset) or of a length-R vector (A^H u): 2 max(N, R) + 2 c64
    w_vf.ensure(sizeof(float2) * (2 * (size_t)std::max(n, R) + 2));
    size_t part = std::max(sizeof(float2) * (size_t)gemv_h_splits(R, n), sizeof(double2) * (size_t)gemv_h_f64_splits(R, n));
    part = std::max(part, sizeof(float2) * (size_t)normal_op_clusters(n));
    w_part.ensure(part * n);
    w_scal.ensure(sizeof(double) * 8);
    d_status.ensure(4 * sizeof(int));
    int *op_status = d_status.as<int>();
    CUDA_TRY(cudaMemsetAsync(op_status, 0, sizeof(int), stream));
    w_ap.ensure(sizeof(double2) * 3 * (size_t)(m + 1) * std::max(1, arnoldi_step_blocks()));
    double2 *V = w_V.as<double2>();
    double *scal = w_scal.as<double>();
    int total_it = 0, max_ref = 0, all_conv = 1;
    double worst = 0.0;
    auto read_scalar = [&](int i) {
        CUDA_TRY(cudaMemcpyAsync(h_pinned + i, scal + i, sizeof(double), cudaMemcpyDeviceToHost, stream));
        CUDA_TRY(cudaStreamSynchronize(stream));
        return h_pinned[i];
    };
    for (int s = 0; s < S; s++) {
        const double2 *b = d_B.as<double2>() + (size_t)s * R;
        double2 *x = d_x.as<double2>() + (size_t)s * n;
        launch_zero_f64(n, x, stream);
        // g0 = A^H b only starts the first inner solve from x = 0, to a relative
        // tolerance far above FP32 rounding, and scales the stopping test; every
        // later A^H r is FP64-accurate, so for c64 A the single-pass FP32
        // product suffices here (the refined solution does not depend on it)
        if (prec == BEM_PREC_C64) {
            // b rounded to c64 once (not once per row and thread inside the product)
            launch_to_c64(R, b, w_vf.as<float2>(), stream);
            launch_gemv_h_c64(R, n, A, lda, w_vf.p, 0, w_gv.p, 1, w_part.p, stream);
        }
        else
            launch_gemv_h_f64(prec, R, n, A, lda, b, w_gv.as<double2>(), w_part.as<double2>(), w_vf.as<float2>(),
                              stream);
        launch_nrm2(n, w_gv.as<double2>(), scal + 0, w_part.as<double>(), stream);
        // |A^H b| reaches the host with the first inner step's result (no wait
        // of its own); a zero right-hand side is recognised there
        CUDA_TRY(cudaMemcpyAsync(h_pinned + 0, scal + 0, sizeof(double), cudaMemcpyDeviceToHost, stream));
        double bn = -1.0;
        bool zero_rhs = false;
        double rel = 1.0;
        bool conv = false;
        int ref = 0;
        for (;; ref++) {
            // With x = 0 (the first step) r = b and g = A^H b, already in w_gv.
            double gn = bn;
            if (ref > 0) {
                launch_resid(prec, R, n, A, lda, x, b, w_r.as<double2>(), w_vf.as<float2>(), stream);
                launch_gemv_h_f64(prec, R, n, A, lda, w_r.as<double2>(), w_gv.as<double2>(),
                                  w_part.as<double2>(), w_vf.as<float2>(), stream);
                launch_nrm2(n, w_gv.as<double2>(), scal + 1, w_part.as<double>(), stream);
                gn = read_scalar(1);
            } else {
                CUDA_TRY(cudaMemcpyAsync(scal + 1, scal + 0, sizeof(double), cudaMemcpyDeviceToDevice, stream));
            }
            rel = ref > 0 ? gn / bn : 1.0;
            if (!std::isfinite(rel)) {
                // a normal-operator launch that gave up on a copy explains it
                if (normal_op_timed_out(op_status, stream))
                    BEM_FAIL(BEM_ERR_TIMEOUT, "normal operator: a bulk copy of A did not complete in time");
                BEM_FAIL(BEM_ERR_NUMERIC, "refinement residual is not finite");
            }
            if (rel <= opt.tol) { conv = true; break; }
            if (ref >= opt.max_refine) break;
            // Inner GMRES on A^H A d = g, d accumulated into x.
            launch_scale_copy(n, w_gv.as<double2>(), scal + 1, V, stream, w_vf.as<float2>(), Vff, w_g.as<double2>(),
                              m + 1);
            // One GMRES step: w = A^H A v_j (c64 copy of v_j; one pass over A
            // when a cluster covers N), the Arnoldi step and Givens rotation,
            // then the residual estimate to h_pinned[4 + (j & 1)], signalled by
            // ev_res[j & 1].
            auto launch_step = [&](int j) {
                // the normal operator's cluster partials are summed by the
                // Arnoldi step itself (one launch less per iteration)
                int nsplit = 0;
                const bool fused = launch_normal_op(R, n, A, lda, w_vf.as<float2>(), w_w.as<double2>(),
                                                    w_part.as<float2>(), op_status, stream, &nsplit);
                if (!fused) {
                    launch_gemv_c64(R, n, A, lda, w_vf.p, 0, w_t.p, 0, stream);              // t = A v_j
                    launch_gemv_h_c64(R, n, A, lda, w_t.p, 0, w_w.p, 1, w_part.p, stream);  // w = A^H t
                }
                const float2 *wpart = fused ? w_part.as<float2>() : nullptr;
                const bool stepped = launch_arnoldi_step(n, j, V, n, Vff, w_w.as<double2>(), w_vf.as<float2>(),
                                                         w_h1.as<double2>(), w_h2.as<double2>(), w_H.as<double2>(),
                                                         ldh, w_cs.as<double2>(), w_sn.as<double2>(),
                                                         w_g.as<double2>(), scal + 3, w_ap.as<double2>(), stream,
                                                         wpart, nsplit);
                if (!stepped && fused) launch_normal_op_sum(n, nsplit, w_part.as<float2>(), w_w.as<double2>(), stream);
                if (!stepped) {
                    launch_dots(n, j + 1, V, n, w_w.as<double2>(), w_h1.as<double2>(), nullptr, stream);
                    launch_update(n, j + 1, V, n, w_h1.as<double2>(), w_w.as<double2>(), stream);
                    launch_dots(n, j + 1, V, n, w_w.as<double2>(), w_h2.as<double2>(), nullptr, stream);
                    launch_update(n, j + 1, V, n, w_h2.as<double2>(), w_w.as<double2>(), stream);
                    launch_nrm2(n, w_w.as<double2>(), scal + 2, nullptr, stream);
                    launch_hcol_finish(j, w_h1.as<double2>(), w_h2.as<double2>(), scal + 2, w_H.as<double2>(), ldh,
                                       stream);
                    launch_scale_copy(n, w_w.as<double2>(), scal + 2, V + (size_t)(j + 1) * n, stream,
                                      w_vf.as<float2>(), Vff + (size_t)(j + 1) * n);
                    launch_givens(j, w_H.as<double2>(), ldh, w_cs.as<double2>(), w_sn.as<double2>(),
                                  w_g.as<double2>(), scal + 3, stream);
                }
                CUDA_TRY(cudaMemcpyAsync(h_pinned + 4 + (j & 1), scal + 3, sizeof(double), cudaMemcpyDeviceToHost,
                                         stream));
                CUDA_TRY(cudaEventRecord(ev_res[j & 1], stream));
            };
            // While the previous estimate is well above the tolerance, step
            // j + 1 is launched before step j's estimate is read, so the host
            // round trip overlaps the GPU.  Should step j be the last after
            // all, step j + 1 has only written basis vector j + 2, Hessenberg
            // column j + 1, rotation j + 1 and g[j + 1], g[j + 2], none of
            // which the solution over the first j + 1 columns reads.
            // "Well above": step j's estimate, extrapolated from the last two
            // at their rate of decrease, still kSpeculate times the tolerance.
            constexpr double kSpeculate = 2.5;
            int jdone = 0;
            double prev = 1.0, prev2 = 1.0;   // estimates / |g| of the last two steps (1 before the first)
            launch_step(0);
            for (int j = 0; j < m; j++) {
                const double rate = std::min(1.0, prev2 > 0.0 ? prev / prev2 : 1.0);
                const bool ahead = j + 1 < m && prev * rate > kSpeculate * opt.inner_tol;
                if (ahead) launch_step(j + 1);
                CUDA_TRY(cudaEventSynchronize(ev_res[j & 1]));
                if (bn < 0.0) {   // the first step of the first inner solve
                    bn = gn = h_pinned[0];
                    if (!(bn > 0.0)) {
                        zero_rhs = true;   // x stays zero
                        break;
                    }
                }
                const double res = h_pinned[4 + (j & 1)];
                jdone = j + 1;
                if (!(res / gn > opt.inner_tol)) break;
                prev2 = prev;
                prev = res / gn;
                if (!ahead && j + 1 < m) launch_step(j + 1);
            }
            if (zero_rhs) break;
            launch_trisolve(jdone, w_H.as<double2>(), ldh, w_g.as<double2>(), w_y.as<double2>(), stream);
            launch_axpy_combo(n, jdone, V, n, w_y.as<double2>(), x, stream);
            total_it += jdone;
        }
        if (bn < 0.0) {   // no inner step ran (max_refine = 0): read |A^H b| now
            bn = read_scalar(0);
            zero_rhs = !(bn > 0.0);
        }
        if (zero_rhs) continue;
        max_ref = std::max(max_ref, ref);
        worst = std::max(worst, rel);
        all_conv &= conv ? 1 : 0;
    }
    CUDA_TRY(cudaStreamSynchronize(stream));
    if (normal_op_timed_out(op_status, stream))
        BEM_FAIL(BEM_ERR_TIMEOUT, "normal operator: a bulk copy of A did not complete in time");
    if (info) {
        info->iterations = total_it;
        info->refinements = max_ref;
        info->rel_residual = worst;
        info->converged = all_conv;
    }
}

void bem_solver_s::eval_field(const double *pts, int P, void *out, int ldo, int precision,
                              const void *u_dev, int u_prec) {
    if (E == 0 || S == 0) BEM_FAIL(BEM_ERR_STATE, "field evaluation needs geometry and sources");
    if (!u_dev && !solved) BEM_FAIL(BEM_ERR_STATE, "no surface solution");
    BEM_CHECK_ARG(P >= 1 && pts && out && ldo >= P, "bad field point arguments");
    ensure_quadrature(opt.order);
    ensure_geo();
    // Field precision follows the assembly precision (c64: FP32 quadrature).
    const int fprec = (prec == BEM_PREC_C128) ? BEM_PREC_C128 : BEM_PREC_C64;
    std::vector<float4> rf(2 * (size_t)P);
    for (int i = 0; i < P; i++) {
        float hx = (float)pts[3 * i], hy = (float)pts[3 * i + 1], hz = (float)pts[3 * i + 2];
        rf[2 * i] = make_float4(hx, hy, hz, 0.f);
        rf[2 * i + 1] = make_float4((float)(pts[3 * i] - hx), (float)(pts[3 * i + 1] - hy), (float)(pts[3 * i + 2] - hz), 0.f);
    }
    f_rows_f.ensure(sizeof(float4) * 2 * (size_t)P);
    f_rows_d.ensure(sizeof(double) * 3 * (size_t)P);
    CUDA_TRY(cudaMemcpyAsync(f_rows_f.p, rf.data(), sizeof(float4) * 2 * (size_t)P, cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaMemcpyAsync(f_rows_d.p, pts, sizeof(double) * 3 * (size_t)P, cudaMemcpyHostToDevice, stream));
    // Surface values in the field precision.
    const void *u = u_dev ? u_dev : d_x.p;
    int uprec = u_dev ? u_prec : BEM_PREC_C128;
    if (uprec != fprec) {
        f_u.ensure((fprec == BEM_PREC_C64 ? sizeof(float2) : sizeof(double2)) * (size_t)N * S);
        if (fprec == BEM_PREC_C64) launch_cast(N * S, (const double2 *)u, f_u.as<float2>(), stream);
        else launch_cast_up(N * S, (const float2 *)u, f_u.as<double2>(), stream);
        u = f_u.p;
    }
    int nsplit = std::max(1, std::min(64, (4 * device_sm_count() + P - 1) / P));
    nsplit = std::min(nsplit, std::max(1, E / 256));
    f_part.ensure(sizeof(double2) * (size_t)nsplit * P * S);
    f_near.ensure(sizeof(double2) * (size_t)P * S);
    f_out.ensure(sizeof(double2) * (size_t)P * S);
    RowPoints rp{f_rows_f.as<float4>(), f_rows_d.as<double>(), P};
    Physics ph = physics();
    if (!assembled) ph.k = k;
    launch_field(fprec, rp, geo_tables(), ph, u, N, S, d_srcs.as<DevSource>(), f_part.as<double2>(), nsplit,
                 f_near.as<double2>(), f_out.as<double2>(), stream);
    std::vector<double2> h((size_t)P * S);
    CUDA_TRY(cudaMemcpyAsync(h.data(), f_out.p, sizeof(double2) * h.size(), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    for (int s = 0; s < S; s++)
        for (int p = 0; p < P; p++) {
            double2 v = h[(size_t)s * P + p];
            if (precision == BEM_PREC_C64) {
                ((float *)out)[2 * ((size_t)s * ldo + p)] = (float)v.x;
                ((float *)out)[2 * ((size_t)s * ldo + p) + 1] = (float)v.y;
            } else {
                ((double *)out)[2 * ((size_t)s * ldo + p)] = v.x;
                ((double *)out)[2 * ((size_t)s * ldo + p) + 1] = v.y;
            }
        }
}
