// Launch wrappers of the box-QP kernels (definitions in kernels.cu).
#pragma once
#include "engine.cuh"

namespace bqp {

// Computes each tile kernel's full wave (SMs x resident blocks per SM); returns the largest.
// Call once before launching.  The `grid` argument of the launchers below is a cap: each
// kernel launches min(cap, its own full wave) blocks.
int tile_grid(int sms);
// resident blocks of the CG product kernel (after tile_grid)
int cg_matvec_slots();
// Tile kernels: grid-stride over the tile table (the grid size is fixed at capture).
void launch_check(const View& v, int grid, cudaStream_t s);
// Step j of a body: the step kernel of one group (step_group(precision, variant)) over the group's
// tiles, or the FP64_EXACT step over the whole table.
void launch_step_group(const View& v, int group, int j, int grid, cudaStream_t s);
void launch_step_exact(const View& v, int j, int grid, cudaStream_t s);
void launch_polish_init(const View& v, int grid, cudaStream_t s);
void launch_polish_residual(const View& v, int grid, cudaStream_t s);
void launch_cg_matvec(const View& v, int grid, cudaStream_t s);
// cap > 0 (inside a graph): also sets cg_loop, the WHILE handle of the CG loop, allowing at
// most `cap` iterations per body.  cap = 0: no handle is touched (host-driven launches).
void launch_cg_vector(const View& v, int grid, cudaStream_t s, cudaGraphConditionalHandle cg_loop = 0, int cap = 0);
// Single-block control kernels that steer the conditional graph nodes.
// fista[k]: handle of the IF node of the precision-k step launches; polish: the IF node of the
// polish branch; cg_loop: the WHILE node of its CG loop.  `steps.n[k]`: kernels inside the
// precision-k FISTA body (steps per body x step groups launched).
struct StepLaunches {
    int n[3];
};
void launch_gate(const View& v, const cudaGraphConditionalHandle* fista, cudaGraphConditionalHandle polish,
                 cudaGraphConditionalHandle cg_loop, StepLaunches steps, int body_steps, cudaStream_t s);
// `steps`: step launches per body; FISTA-phase instances advance it_cur by up to that many.
void launch_control(const View& v, cudaGraphConditionalHandle loop, int steps, cudaStream_t s);
// Host-driven variants of the control kernels (no conditional handles).
void launch_gate_plain(const View& v, int steps, cudaStream_t s);
void launch_control_plain(const View& v, int steps, cudaStream_t s);
// Admission, first kernel: the convexity gate and Gershgorin bound of the uploaded full CSR
// (FP64 values `val`) into *rec.gate (cleared first), the FP64 diagonal into rec.diag and, for the
// mixed engine, the hi/lo FP32 values into rec.vhi/rec.vlo.  The later admission kernels read L there.
void launch_gate(const InstDev& rec, int64_t n, const double* val, cudaStream_t s);
// The same pass on raw device pointers (diag, vhi, vlo may be null: not stored).
void launch_gate_raw(int64_t n, const int32_t* rowptr, const int32_t* col, const double* val, GateResult* out,
                     double* diag, float* vhi, float* vlo, cudaStream_t s);
// Admission, mixed engine, after launch_gate on the same stream: 1/diag, preconditioner scales and
// the FP32 cost and bounds (nothing for the FP64 engines).
// The record is passed by value: the instance is installed in its slot later, between graph launches.
void launch_prepare_instance(const InstDev& rec, int64_t n, cudaStream_t s);
// Mixed engine: per-row FISTA steps (diagonally preconditioned when `scaled`, else 1/L), after
// launch_prepare_instance on the same stream; val = the FP64 values.  With rec.lip_device the
// power estimate replaces the Gershgorin bound (power_scratch: power_scratch_bytes()).
void launch_precondition(const InstDev& rec, int64_t n, const double* val, bool scaled, void* power_scratch,
                         cudaStream_t s);
// BQP_LIPSCHITZ_POWER: Lanczos on the power iteration's Krylov space of S Q S (S = diag(rec.s)
// when `scaled`), FP64, at admission; *rec.lprec holds the Gershgorin bound of that matrix before
// and the estimate after.  scratch: power_scratch_bytes(n) bytes of device memory, 256-aligned.
size_t power_scratch_bytes(int64_t n);
void launch_power_lipschitz(const InstDev& rec, int64_t n, const double* val, bool scaled, void* scratch, cudaStream_t s);
// Admission: x0 = clip(0, l, u), w = x0, start clock; one instance.
// Re-arm of resident solves: records staged on the device, spans (staged index, first row) of
// kRearmRows rows each, one block per span.
void launch_rearm(const View& v, const InstDev* stage, const int32_t* slots, const int2* spans, int n_spans,
                  cudaStream_t s);
void launch_init_instance(const View& v, int slot, int n, int precision, cudaStream_t s);

// Standalone FP64 check on caller device arrays (one instance, block partials in scratch).
// scratch must hold check_scratch_bytes(n) bytes.
size_t check_scratch_bytes(int64_t n);
int check_grid(int64_t n);
void launch_check_standalone(int64_t n, const int32_t* rowptr, const int32_t* col, const double* val,
                             const double* x, const double* c, const double* l, const double* u,
                             double tol, double offset, int gate, void* scratch, double* result,
                             cudaStream_t s);
// Loads the standalone check kernel into the current context now (under lazy module loading
// its first launch would load it) and opts it into its shared-memory size.
cudaError_t load_check_standalone();

// Plugin-level FISTA step (reference numerics: FP64, division by L, no FMA), ping-pong w.
void launch_box_step(int64_t n, const int32_t* rowptr, const int32_t* col, const double* val,
                     const double* c, const double* l, const double* u, double L, double beta,
                     double* x, const double* w_in, double* w_out, cudaStream_t s);

}  // namespace bqp
