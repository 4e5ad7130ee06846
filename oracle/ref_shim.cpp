// ORACLE -- test infrastructure only (the reference itself, compiled from its sources).
//
// Compiles the reference translation unit reproducer.cpp unchanged (with
// PRIMORDIAL_ROS2S_NO_MAIN, reproducer.cpp:8590) and exposes its functions through
// a C ABI with the same signatures as wr_oracle.cpp's wro_* entry points, so the
// oracle restatement can be checked bit for bit against the reference's own code.
// The gridwide-independent policy exists in the reference only as CUDA kernels
// (reproducer.cpp:7696-7785); wrr_prepare / wrr_advance run those kernel bodies
// as host loops that call the reference's own helper functions.
//
// Built only where the reference tree is present, by oracle/build_ref.sh, into
// oracle/_ref/ (never committed, never shipped as product).
#define PRIMORDIAL_ROS2S_NO_MAIN 1
#include REFERENCE_TU
#include <atomic>
#include <cfloat>
#include <cstring>
#include "../include/warp_reactor.h"

static_assert(sizeof(CollapseState) == sizeof(wr_collapse_state), "layout");

namespace {
void cas(std::atomic<int>& f, int v) { int e = 1; f.compare_exchange_strong(e, v); }
}

extern "C" {

void wrr_make_collapse_state(wr_collapse_state* out) {
    pc::set_redshift(30.0);
    CollapseState c = make_collapse_state();
    std::memcpy(out, &c, sizeof(c));
}

void wrr_rhs(const double* y, double* dydt) {
    pc::set_redshift(30.0);
    pc::PrimordialChem::state_type ys;
    pc::PrimordialChem::rhs_type out;
    for (int i = 0; i < 15; ++i) ys[i] = y[i];
    pc::PrimordialChem::rhs(0.0, ys, out);
    for (int i = 0; i < 15; ++i) dydt[i] = out[i];
}

void wrr_jac(const double* y, double* J) {
    pc::set_redshift(30.0);
    pc::PrimordialChem::state_type ys;
    pc::PrimordialChem::jacobian_type jac;
    for (int i = 0; i < 15; ++i) ys[i] = y[i];
    pc::PrimordialChem::jacobian(0.0, ys, jac);
    for (int r = 0; r < 15; ++r)
        for (int c = 0; c < 15; ++c) J[r * 15 + c] = jac[r][c];
}

// actual_rhs / actual_jac at a given burn state (X, T) without flooring or EOS
void wrr_net_rhs(const double* X, double T, double* f) {
    pc::set_redshift(30.0);
    pc::burn_t s{};
    s.T = T;
    for (int i = 0; i < 14; ++i) s.xn[i] = X[i];
    pc::Array1D<integrators::Real, 1, pc::neqs> ydot;
    pc::actual_rhs(s, ydot);
    for (int i = 0; i < 15; ++i) f[i] = ydot(i + 1);
}

void wrr_net_jac(const double* X, double T, double* J, double* f) {
    pc::set_redshift(30.0);
    pc::burn_t s{};
    s.T = T;
    for (int i = 0; i < 14; ++i) s.xn[i] = X[i];
    pc::PrimordialChem::jacobian_type jac;
    for (auto& row : jac) row.fill(0.0);
    pc::JacobianAdapter adapter{jac};
    pc::actual_jac(s, adapter);
    for (int r = 0; r < 15; ++r)
        for (int c = 0; c < 15; ++c) J[r * 15 + c] = jac[r][c];
    wrr_net_rhs(X, T, f);
}

int wrr_lu(double* A, int* ipvt) {
    std::array<std::array<double, 15>, 15> M;
    std::array<int, 15> ip;
    for (int r = 0; r < 15; ++r)
        for (int c = 0; c < 15; ++c) M[r][c] = A[r * 15 + c];
    const int info = integrators::linalg::lu_decomposition<15>(M, ip);
    for (int r = 0; r < 15; ++r)
        for (int c = 0; c < 15; ++c) A[r * 15 + c] = M[r][c];
    for (int i = 0; i < 15; ++i) ipvt[i] = ip[i];
    return info;
}

void wrr_lu_solve(const double* LU, const int* ipvt, double* x) {
    std::array<std::array<double, 15>, 15> M;
    std::array<int, 15> ip;
    std::array<double, 15> v;
    for (int r = 0; r < 15; ++r)
        for (int c = 0; c < 15; ++c) M[r][c] = LU[r * 15 + c];
    for (int i = 0; i < 15; ++i) { ip[i] = ipvt[i]; v[i] = x[i]; }
    integrators::linalg::lu_solve<15>(M, ip, v);
    for (int i = 0; i < 15; ++i) x[i] = v[i];
}

int wrr_burn(wr_collapse_state* cell, double dt) {
    pc::set_redshift(30.0);
    CollapseState* c = reinterpret_cast<CollapseState*>(cell);
    return static_cast<int>(burn_ros2s(c->current, dt, c->stats));
}

int wrr_prepare(wr_collapse_state* cells_, int n, int cgs, double grid_time, int step,
                int perturb, double* dt_grid_out, int nthreads) {
    pc::set_redshift(30.0);
    CollapseState* cells = reinterpret_cast<CollapseState*>(cells_);
    std::atomic<int> failure{1};
    std::vector<double> cand(static_cast<size_t>(n));
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
    for (int cell = 0; cell < n; ++cell) {  // body of reproducer.cpp:7702-7733
        cand[cell] = DBL_MAX;
        if (failure.load() != 1) continue;
        CollapseState& state = cells[cell];
        if (state.completed_steps < cgs) continue;
        if (state.completed_steps != cgs || state.time != grid_time) { cas(failure, -1); continue; }
        apply_perturbation(state, cell, step, perturb != 0);
        const double dt = collapse_timestep(state);
        if (!valid_positive(dt) || !valid_positive(state.density_driver)) { cas(failure, -1); continue; }
        if (dt < 10.0) {
            const double tff = dt / tff_reduc;
            state.density_driver += dt * (state.density_driver / tff);
            continue;
        }
        cand[cell] = dt;
    }
    double dt_grid = DBL_MAX;
    for (double c : cand) if (c < dt_grid) dt_grid = c;
    *dt_grid_out = dt_grid;
    return failure.load();
}

int wrr_advance(wr_collapse_state* cells_, int n, int cgs, double next_grid_time,
                double dt_grid, int* integrated, int nthreads) {
    pc::set_redshift(30.0);
    CollapseState* cells = reinterpret_cast<CollapseState*>(cells_);
    std::atomic<int> failure{1};
    int count = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : count) num_threads(nthreads > 0 ? nthreads : 1)
    for (int cell = 0; cell < n; ++cell) {  // body of reproducer.cpp:7742-7784
        if (failure.load() != 1) continue;
        CollapseState& state = cells[cell];
        if (state.completed_steps != cgs) continue;
        const double local_dt = collapse_timestep(state);
        if (local_dt < 10.0) continue;
        const double old_density = state.density_driver;
        const double tff = local_dt / tff_reduc;
        state.density_driver += dt_grid * (state.density_driver / tff);
        if (!valid_positive(state.density_driver) || state.density_driver > 2.0e-6) continue;
        const double density_ratio = state.density_driver / old_density;
        for (auto& xn : state.current.xn) xn *= density_ratio;
        state.current.rho *= density_ratio;
        const auto result = burn_ros2s(state.current, dt_grid, state.stats);
        if (result != integrators::IntegratorResult::SUCCESS) { cas(failure, static_cast<int>(result)); continue; }
        pc::floor_and_normalize_number_densities(state.current);
        pc::balance_charge(state.current);
        pc::floor_and_normalize_number_densities(state.current);
        pc::eos_re(state.current);
        state.time = next_grid_time;
        state.completed_steps = cgs + 1;
        count += 1;
    }
    *integrated = count;
    return failure.load();
}

// Host loop of run_cells_cuda, reproducer.cpp:7859-7959.
int wrr_run(wr_collapse_state* cells, int n, int perturb, int* cgs, int max_steps, int nthreads) {
    int result = 1;
    double grid_time = 0.0;
    const int steps = max_steps > 0 ? max_steps : max_collapse_steps;
    for (int step = 0; result == 1 && step < steps; ++step) {
        double dt_grid = DBL_MAX;
        result = wrr_prepare(cells, n, *cgs, grid_time, step, perturb, &dt_grid, nthreads);
        if (result != 1) break;
        if (dt_grid == DBL_MAX) break;
        const double next = grid_time + dt_grid;
        if (!valid_positive(dt_grid) || !std::isfinite(next)) { result = -1; break; }
        int integrated = 0;
        result = wrr_advance(cells, n, *cgs, next, dt_grid, &integrated, nthreads);
        if (result != 1) break;
        if (integrated == 0) break;
        grid_time = next;
        *cgs += 1;
    }
    return result;
}

}  // extern "C"
