// Native step driver of the mixed-precision Newton solver: the control flow of
// NewtonBonds.step and fgmres (experiments/bonded_dem_newton.py:13-60,
// 132-201) as host code that launches this library's entry points directly.
//
// The Python control path (MixedNewtonBonds.step) and this driver issue the
// same entry points in the same order with the same arguments, and take the
// same host decisions in float64 (Givens rotations with hypot, back
// substitution, convergence tests, Armijo line search), so a step gives
// bit-identical results either way.  What changes is the host cost between
// launches: a few microseconds of C++ instead of Python, which matters after
// each of the step's small device reads (the FGMRES Hessenberg column, the
// residual norms), when the GPU idles until the next launch arrives.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "dpf_gb300.h"

namespace dpf {
namespace driver {

// max over sites of |y_w| (the rotation part of the increment); non-negative
// doubles order like their bit patterns, so an integer atomicMax is exact.
__global__ void max_rotation_kernel(int64_t n, const double *y, unsigned long long *out) {
    double best = 0.0;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
        const double *w = y + 6 * s + 3;
        const double v = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        best = v > best ? v : best;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double other = __shfl_xor_sync(0xffffffffu, best, o);
        best = other > best ? other : best;
    }
    if ((threadIdx.x & 31) == 0 && best > 0.0) atomicMax(out, (unsigned long long)__double_as_longlong(best));
}

// launch categories timed with step->timing (the order of DPF_NEWTON_TIMERS)
enum Timer {
    kSetup = 0,  // float64 setup or the per-step begin
    kResidual,   // residual bond and site passes
    kScaling,    // 6x6 blocks and their inverses
    kPcg,        // the elastic PCG
    kJvp,        // J d
    kCommit,     // end state of the accepted increment
    kPack,       // bond-end records of a tangent
    kKrylov,     // Arnoldi, row combination, Krylov norms and scaling
    kNorms,      // scaled residual and its norms
    kVector,     // float64 vector updates (rhs, correction, candidates, float32 copies)
    kAccept      // velocity, rotation, work and step statistics
};
static_assert(kAccept + 1 == DPF_NEWTON_TIMERS, "one timer per category");

// CUDA events around the launches (only with step->timing), created for the
// call and destroyed before it returns.
struct Timing {
    bool on = false;
    cudaStream_t stream = nullptr;
    std::vector<int> keys;
    std::vector<cudaEvent_t> events;
    void record(bool opening, int key) {
        if (!on) return;
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) != cudaSuccess) {
            on = false;  // no timing rather than a failed step
            return;
        }
        if (opening) keys.push_back(key);
        events.push_back(e);
        cudaEventRecord(e, stream);
    }
    // after the stream has been synchronised
    void collect(dpf_newton_info *info) {
        for (size_t k = 0; k < keys.size() && 2 * k + 1 < events.size(); ++k) {
            float ms = 0.0f;
            if (cudaEventElapsedTime(&ms, events[2 * k], events[2 * k + 1]) == cudaSuccess) {
                info->time_ms[keys[k]] += ms;
                info->timed_launches[keys[k]] += 1;
            }
        }
    }
    ~Timing() {
        for (cudaEvent_t e : events) cudaEventDestroy(e);
    }
};

struct Step {
    const dpf_mixed_newton *s;
    const dpf_newton_step *a;
    dpf_newton_info *info;
    cudaStream_t st;
    int64_t n, n6, m;
    double *y, *cand, *r, *r_cand, *scaled, *rhs, *x, *res, *corr, *ax;
    double *host;     // pinned: [0..8) scalars, [8..10) scales, [12] a norm, [16..80) h column
    int *host_int;    // pinned ints after the doubles: [0] status, [1] inner
    Timing timing;
    bool packed = false;
    double rhs_scale = -1.0;
    // the iterate's 6x6 blocks, their inverses and units, and the other set,
    // which the speculative scaling of a line-search candidate writes
    struct Scaling {
        float *block32, *p32, *units32;
        double *units;
    } cur, alt;

    // one library call of `kernels` launches, timed under `key`
    template <class F>
    int call(int key, int kernels, F &&f) {
        timing.record(true, key);
        const int rc = f();
        timing.record(false, key);
        if (!rc) info->launches += kernels;
        return rc;
    }

    // copy `count` device scalars (and optionally the status word and the
    // step's scales) to pinned memory, then wait for the stream
    int fetch(int count, bool status, bool scales) {
        if (count && cudaMemcpyAsync(host, s->scalars, count * sizeof(double), cudaMemcpyDeviceToHost, st))
            return DPF_ERR_CUDA;
        if (status && cudaMemcpyAsync(host_int, s->status, sizeof(int), cudaMemcpyDeviceToHost, st))
            return DPF_ERR_CUDA;
        if (scales && cudaMemcpyAsync(host + 8, s->scales, 2 * sizeof(double), cudaMemcpyDeviceToHost, st))
            return DPF_ERR_CUDA;
        return cudaStreamSynchronize(st) == cudaSuccess ? DPF_OK : DPF_ERR_CUDA;
    }

    int residual(const double *yy, double *out, bool use_p) {
        int rc = call(kVector, 1, [&] { return dpf_to_float(n6, yy, s->y32, st); });
        if (rc) return rc;
        if (cudaMemsetAsync(s->status, 0, sizeof(int), st)) return DPF_ERR_CUDA;
        return call(kResidual, m ? 2 : 1, [&] {
            return dpf_mixed_residual(s->graph, s->bond_data, yy, s->y32, s->mass, s->fixed, a->dt, s->r0, 1,
                                      use_p ? cur.p32 : nullptr, use_p ? cur.units32 : nullptr, out, nullptr,
                                      use_p ? s->scalars : nullptr, s->wrench32, s->partials, s->status, st);
        });
    }

    // blocks and scaling of the tangent in bond_data into `into`, then the
    // scaled residual of rr and its norms [|r|, max |s|, |s|] into norms
    int scaling_norms(const Scaling &into, const double *rr, double *norms) {
        int rc = call(kScaling, 1, [&] {
            return dpf_mixed_scaling(s->graph, s->bond_data, s->mass32, s->fixed, s->radii, a->dt, into.block32,
                                     into.p32, into.units, into.units32, st);
        });
        if (rc) return rc;
        return call(kNorms, 1, [&] {
            return dpf_mixed_scale_residual(n, into.p32, into.units32, rr, scaled, norms, s->partials, st);
        });
    }

    // the elastic PCG on a float32 Krylov vector
    int precondition(const float *vector, float *out) {
        if (!packed) {
            const int rc = call(kPack, 2, [&] {
                return dpf_end_pack(s->graph, s->bond_data, 0.25 * a->dt * a->dt, cur.p32, s->mass32, s->fixed,
                                    s->ends, s->p24, s->site4, st);
            });
            if (rc) return rc;
            packed = true;
        }
        return call(kPcg, 1, [&] {
            return dpf_end_precondition_f32(s->graph, s->ends, s->site4, s->fixed, cur.block32, s->p24, cur.units32,
                                            vector, 0.03, 80, out, s->inner, s->end_workspace, s->end_partials,
                                            s->barrier, s->status, s->end_variant, st);
        });
    }

    // J d on float32 Krylov vectors
    int jvp32(const float *direction, float *out) {
        return call(kJvp, m ? 3 : 2, [&] {
            return dpf_mixed_jacobian_vector_f32(s->graph, s->bond_data, s->y32, direction, s->mass32, s->fixed,
                                                 a->dt, cur.units32, cur.p32, out, s->d32, s->wrench32, st);
        });
    }

    // J d on a float64 vector (the Newton direction)
    int jvp(const double *direction, double *out) {
        return call(kJvp, m ? 3 : 2, [&] {
            return dpf_mixed_jacobian_vector(s->graph, s->bond_data, s->y32, direction, s->mass32, s->fixed, a->dt,
                                             cur.units32, cur.p32, out, s->d32, s->wrench32, nullptr, nullptr, st);
        });
    }

    // One restart cycle of the right-preconditioned FGMRES with CGS2 Arnoldi
    // (MixedNewtonBonds._fgmres32 in newton.py) from `start` with |start| = g0:
    // x += the cycle's correction, then J x (from the kept products J z_k), the
    // true residual res = rhs - J x and its norm (krylov_scalars[1]) are
    // enqueued but not read: the caller fetches that norm together with the
    // speculative line-search values.  The Krylov vectors are float32 (the PCG
    // and JVP outputs carry float32 precision), their sums exact float32
    // pairs; x, rhs and the true residual are float64.  *krylov counts the
    // Arnoldi steps; *singular reports a zero Givens denominator.
    int fgmres_cycle(const double *start, double g0, double norm, double tolerance, int width, int *krylov,
                     bool *singular) {
        *singular = false;
        if (width > s->krylov_width) return DPF_ERR_ARGUMENT;
        const int ldh = width;  // H is (width + 1) x width, row-major
        double H[64 * 63];
        double cs[64], sn[64], g[65], coef[64];
        std::memset(H, 0, sizeof(double) * (width + 1) * width);
        std::memset(cs, 0, sizeof(double) * width);
        std::memset(sn, 0, sizeof(double) * width);
        std::memset(g, 0, sizeof(double) * (width + 1));
        g[0] = g0;
        int rc = call(kKrylov, 1, [&] { return dpf_scale_to_float(n6, 1.0 / g[0], start, s->basis, st); });
        if (rc) return rc;
        for (int j = 0; j < width; ++j) {
            float *bj = s->basis + (int64_t)j * n6;
            float *tj = s->transformed + (int64_t)j * n6;
            float *pj = s->products + (int64_t)j * n6;
            rc = precondition(bj, tj);
            if (rc) return rc;
            rc = jvp32(tj, pj);
            if (rc) return rc;
            rc = call(kKrylov, 1, [&] {
                return dpf_arnoldi_cgs2_f32(n6, s->basis, n6, j, pj, s->w32, s->h, s->krylov_partials, s->barrier,
                                            s->status, st);
            });
            if (rc) return rc;
            double *column = host + 16;
            if (cudaMemcpyAsync(column, s->h, (j + 2) * sizeof(double), cudaMemcpyDeviceToHost, st) ||
                cudaStreamSynchronize(st))
                return DPF_ERR_CUDA;
            for (int k = 0; k <= j + 1; ++k) H[k * ldh + j] = column[k];
            const bool breakdown = H[(j + 1) * ldh + j] < 1e-14;
            for (int k = 0; k < j; ++k) {
                const double hk = H[k * ldh + j], hk1 = H[(k + 1) * ldh + j];
                H[k * ldh + j] = cs[k] * hk + sn[k] * hk1;
                H[(k + 1) * ldh + j] = -sn[k] * hk + cs[k] * hk1;
            }
            const double denominator = std::hypot(H[j * ldh + j], H[(j + 1) * ldh + j]);
            if (denominator == 0.0) {
                *singular = true;
                return DPF_OK;
            }
            cs[j] = H[j * ldh + j] / denominator;
            sn[j] = H[(j + 1) * ldh + j] / denominator;
            H[j * ldh + j] = denominator;
            H[(j + 1) * ldh + j] = 0.0;
            const double gj = g[j];
            g[j + 1] = -sn[j] * gj;
            g[j] = cs[j] * gj;
            *krylov += 1;
            if (std::fabs(g[j + 1]) <= tolerance * norm || breakdown || j + 1 == width) {
                // back substitution of the (j+1) x (j+1) upper triangle
                const int k = j + 1;
                for (int i = k - 1; i >= 0; --i) {
                    double acc = g[i];
                    for (int c = i + 1; c < k; ++c) acc -= H[i * ldh + c] * coef[c];
                    coef[i] = acc / H[i * ldh + i];
                }
                rc = call(kKrylov, 1, [&] { return dpf_combine_rows_f32(n6, s->transformed, n6, k, coef, x, st); });
                if (rc) return rc;
                // J x = sum_k c_k J z_k from the stored products (J is linear)
                if (cudaMemsetAsync(ax, 0, n6 * sizeof(double), st)) return DPF_ERR_CUDA;
                rc = call(kKrylov, 1, [&] { return dpf_combine_rows_f32(n6, s->products, n6, k, coef, ax, st); });
                if (rc) return rc;
                rc = call(kVector, 1, [&] { return dpf_axpby(n6, 1.0, rhs, -1.0, ax, res, st); });
                if (rc) return rc;
                return call(kKrylov, 1, [&] {
                    return dpf_dot_norm(n6, res, nullptr, s->krylov_scalars, s->krylov_partials, st);
                });
            }
        }
        return DPF_OK;
    }

    int accept() {
        int rc = call(kVector, 1, [&] { return dpf_to_float(n6, y, s->y32, st); });
        if (rc) return rc;
        const dpf_history &h = a->history;
        rc = call(kCommit, m ? 3 : 1, [&] {
            if (s->history_corrections)
                return dpf_mixed_commit_lazy(s->graph, s->bond_data, h.x, y, s->y32, a->x_end, s->history_corrections,
                                             s->wrench32, s->loads, st);
            return dpf_mixed_commit(s->graph, s->bond_data, &h, y, s->y32, a->x_end, a->normal_end, a->offset_end,
                                    a->fn_end, a->fs_end, a->mt_end, a->mb_end, s->wrench32, s->loads, st);
        });
        if (rc) return rc;
        rc = call(kAccept, 1, [&] { return dpf_accept_step(n, y, a->dt, a->v, a->rotation, st); });
        if (rc) return rc;
        rc = call(kAccept, 1, [&] { return dpf_dot_norm(n6, a->external, y, s->scalars, s->partials, st); });
        if (rc) return rc;
        if (cudaMemsetAsync(s->scalars + 2, 0, sizeof(double), st)) return DPF_ERR_CUDA;
        rc = call(kAccept, 1, [&] {
            const int grid = (int)((n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024);
            max_rotation_kernel<<<grid, 256, 0, st>>>(n, y, reinterpret_cast<unsigned long long *>(s->scalars + 2));
            return cudaGetLastError() == cudaSuccess ? DPF_OK : DPF_ERR_CUDA;
        });
        if (rc) return rc;
        if (cudaMemcpyAsync(host_int + 1, s->inner, sizeof(int), cudaMemcpyDeviceToHost, st)) return DPF_ERR_CUDA;
        rc = fetch(3, false, false);
        if (rc) return rc;
        info->work = host[0];
        info->max_rotation = host[2];
        info->cg_iterations = host_int[1];
        return DPF_OK;
    }

    int run() {
        if (cudaMemsetAsync(s->inner, 0, sizeof(int), st) || cudaMemsetAsync(s->status, 0, sizeof(int), st) ||
            cudaMemsetAsync(y, 0, n6 * sizeof(double), st))
            return DPF_ERR_CUDA;
        if ((a->v_in && cudaMemcpyAsync(a->v, a->v_in, n6 * sizeof(double), cudaMemcpyDeviceToDevice, st)) ||
            (a->rotation_in &&
             cudaMemcpyAsync(a->rotation, a->rotation_in, 9 * n * sizeof(double), cudaMemcpyDeviceToDevice, st)))
            return DPF_ERR_CUDA;
        int rc;
        if (a->refresh) {
            const dpf_history &h = a->history;
            rc = call(kSetup, m ? 2 : 1, [&] {
                return dpf_mixed_setup(s->graph, &s->stiffness, &h, s->mass, a->v, a->external, s->fixed, a->dt,
                                       s->bond_data, s->r0, s->loads, s->scales, s->wrench64,
                                       s->history_corrections, s->partials, s->status, st);
            });
        } else {
            rc = call(kSetup, 1, [&] {
                return dpf_mixed_begin(n, s->loads, s->mass, a->v, a->external, s->fixed, a->dt, s->r0, s->scales,
                                       s->partials, st);
            });
        }
        if (rc) return rc;
        bool cached = false, prefetched = false;
        double pre[3] = {0.0, 0.0, 0.0};
        const double dt = a->dt;
        for (int iteration = 0; iteration <= a->max_iterations; ++iteration) {
            double rnorm, local, merit;
            const bool first = rhs_scale < 0.0;
            if (prefetched) {
                // the accepted candidate's norms came with the line-search fetch
                rnorm = pre[0];
                local = pre[1];
                merit = pre[2];
            } else {
                if (iteration == 0 && a->committed_start && !a->refresh) {
                    if (cudaMemsetAsync(s->status, 0, sizeof(int), st)) return DPF_ERR_CUDA;
                    rc = call(kResidual, 1,
                              [&] { return dpf_mixed_initial_residual(n, s->r0, s->fixed, s->y32, r, st); });
                    if (rc) return rc;
                } else if (!cached) {
                    rc = residual(y, r, false);
                    if (rc) return rc;
                }
                rc = scaling_norms(cur, r, s->scalars);
                if (rc) return rc;
                rc = fetch(3, !cached, first);
                if (rc) return rc;
                const int status = cached ? 0 : host_int[0];
                if (status) {
                    info->outcome = DPF_NEWTON_GUARD;
                    info->guard = status;
                    return DPF_OK;
                }
                rnorm = host[0];
                local = host[1];
                merit = host[2];
            }
            cached = false;
            prefetched = false;
            packed = false;
            if (first) {
                const double sa = host[8], sl = host[9];
                double v = sa;
                if (0.5 * dt * dt * sl > v) v = 0.5 * dt * dt * sl;
                if (1e-30 > v) v = 1e-30;
                rhs_scale = v;
            }
            const double relative = rnorm / rhs_scale;
            info->relative = relative;
            info->local = local;
            info->nonlinear_iterations = iteration;
            if (!std::isfinite(relative) || !std::isfinite(local)) {
                info->outcome = DPF_NEWTON_NONFINITE;
                return DPF_OK;
            }
            if (info->trace_len < DPF_NEWTON_TRACE) {
                info->trace[2 * info->trace_len] = relative;
                info->trace[2 * info->trace_len + 1] = local;
                info->trace_len += 1;
            }
            if (relative < a->tolerance && local < a->pose_tolerance) {
                rc = accept();
                if (rc) return rc;
                info->outcome = DPF_NEWTON_CONVERGED;
                return DPF_OK;
            }
            if (iteration == a->max_iterations) break;
            rc = call(kVector, 1, [&] { return dpf_axpby(n6, -1.0, scaled, 0.0, scaled, rhs, st); });
            if (rc) return rc;
            // FGMRES cycles (restart 32, at most 256 Arnoldi steps).  Each cycle's
            // true-residual norm is fetched together with a speculative first
            // line-search step (factor 1) and the scaling and norms of that
            // candidate, which the next iteration starts from if it is accepted:
            // one wait instead of three.  A failed guess costs work, not results:
            // the iterate's scaling stays in `cur`, and y32 is restored before a
            // restart's JVPs.
            if (cudaMemsetAsync(x, 0, n6 * sizeof(double), st)) return DPF_ERR_CUDA;
            int krylov = 0;
            const double *start = rhs;
            double g0 = merit;
            bool speculated = false;
            for (;;) {
                if (merit != 0.0) {
                    const int width = 256 - krylov < 32 ? 256 - krylov : 32;
                    bool singular;
                    rc = fgmres_cycle(start, g0, merit, a->linear_tolerance, width, &krylov, &singular);
                    if (rc) return rc;
                    if (singular) {
                        info->outcome = DPF_NEWTON_SINGULAR;
                        return DPF_OK;
                    }
                }
                rc = call(kVector, 1, [&] { return dpf_masked_scale(n, x, cur.units, s->fixed, corr, st); });
                if (rc) return rc;
                rc = call(kVector, 1, [&] { return dpf_axpby(n6, 1.0, y, 1.0, corr, cand, st); });
                if (rc) return rc;
                rc = residual(cand, r_cand, true);
                if (rc) return rc;
                rc = scaling_norms(alt, r_cand, s->scalars + 4);
                if (rc) return rc;
                if (merit != 0.0 &&
                    cudaMemcpyAsync(host + 12, s->krylov_scalars + 1, sizeof(double), cudaMemcpyDeviceToHost, st))
                    return DPF_ERR_CUDA;
                if (cudaMemcpyAsync(host + 4, s->scalars + 4, 3 * sizeof(double), cudaMemcpyDeviceToHost, st))
                    return DPF_ERR_CUDA;
                rc = fetch(3, true, false);
                if (rc) return rc;
                const double krylov_relative = merit != 0.0 ? host[12] / merit : 0.0;
                info->krylov_relative = krylov_relative;
                if (krylov_relative <= 1.05 * a->linear_tolerance) {
                    speculated = true;
                    break;
                }
                if (krylov >= 256) {
                    info->outcome = DPF_NEWTON_KRYLOV;
                    return DPF_OK;
                }
                // restart from the true residual; the JVPs need the iterate's y32 again
                rc = call(kVector, 1, [&] { return dpf_to_float(n6, y, s->y32, st); });
                if (rc) return rc;
                start = res;
                g0 = host[12];
            }
            info->krylov_iterations += krylov;
            bool accepted = false;
            for (int power = 0; power < 10; ++power) {
                const double factor = std::ldexp(1.0, -power);
                if (power > 0 || !speculated) {
                    rc = call(kVector, 1, [&] { return dpf_axpby(n6, 1.0, y, factor, corr, cand, st); });
                    if (rc) return rc;
                    rc = residual(cand, r_cand, true);
                    if (rc) return rc;
                    rc = fetch(3, true, false);
                    if (rc) return rc;
                }
                if (host_int[0]) continue;
                if (host[2] < (1.0 - 1e-4 * factor) * merit) {
                    double *t = y;
                    y = cand;
                    cand = t;
                    t = r;
                    r = r_cand;
                    r_cand = t;
                    if (power == 0) {
                        // the next iteration's scaling is the candidate's: swap the sets
                        const Scaling keep = cur;
                        cur = alt;
                        alt = keep;
                        info->scaling_alternate ^= 1;
                        prefetched = true;
                        pre[0] = host[4];
                        pre[1] = host[5];
                        pre[2] = host[6];
                    } else {
                        cached = true;
                    }
                    accepted = true;
                    break;
                }
            }
            if (!accepted) {
                info->outcome = DPF_NEWTON_LINE_SEARCH;
                return DPF_OK;
            }
        }
        info->outcome = DPF_NEWTON_DIVERGED;
        return DPF_OK;
    }
};

}  // namespace driver
}  // namespace dpf

extern "C" int dpf_mixed_newton_step(const dpf_mixed_newton *solver, const dpf_newton_step *step,
                                     dpf_newton_info *info, void *stream) {
    using dpf::driver::Step;
    if (!solver || !step || !info || !solver->graph || solver->graph->n_sites <= 0 || !solver->vectors ||
        !solver->host || !solver->basis || !solver->transformed || !solver->products || !solver->w32 || !solver->h ||
        !solver->block32_b || !solver->p32_b || !solver->units_b || !solver->units32_b ||
        solver->krylov_width < 1 ||
        solver->krylov_width > 62 || !step->external || !step->v || !step->rotation || !(step->dt > 0.0) ||
        step->max_iterations < 0 || ((uintptr_t)solver->vectors & 15u))
        return DPF_ERR_ARGUMENT;
    std::memset(info, 0, sizeof(*info));
    Step run;
    run.s = solver;
    run.a = step;
    run.info = info;
    run.st = (cudaStream_t)stream;
    run.n = solver->graph->n_sites;
    run.n6 = 6 * run.n;
    run.m = solver->graph->n_bonds;
    double *v = solver->vectors;
    double **slots[DPF_NEWTON_VECTORS] = {&run.y, &run.cand, &run.r, &run.r_cand, &run.scaled,
                                          &run.rhs, &run.x, &run.res, &run.corr, &run.ax};
    for (int k = 0; k < DPF_NEWTON_VECTORS; ++k) *slots[k] = v + (int64_t)k * run.n6;
    run.host = solver->host;
    run.host_int = reinterpret_cast<int *>(solver->host + 96);
    run.cur = {solver->block32, solver->p32, solver->units32, solver->units};
    run.alt = {solver->block32_b, solver->p32_b, solver->units32_b, solver->units_b};
    run.timing.on = step->timing != 0;
    run.timing.stream = run.st;
    const int rc = run.run();
    if (!run.timing.events.empty() && cudaStreamSynchronize(run.st) == cudaSuccess) run.timing.collect(info);
    return rc;
}

extern "C" int dpf_newton_struct_sizes(int64_t *out) {
    if (!out) return DPF_ERR_ARGUMENT;
    out[0] = (int64_t)sizeof(dpf_mixed_newton);
    out[1] = (int64_t)sizeof(dpf_newton_step);
    out[2] = (int64_t)sizeof(dpf_newton_info);
    return DPF_OK;
}
