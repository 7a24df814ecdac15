/*
 * mpmc_gb300_flash.h -- C ABI of the GB300 PR76 two-phase PT flash.
 *
 * This is the drop-in boundary for MPMC_HNU's unified flash backend.  In the
 * reference, callers reach the per-cell flash through the virtual
 *   mpmc::flash::PtFlashBackend::solve(const PtFlashRequest&)
 *     (modules/flash/include/mpmc/flash/pt_flash_backend.hpp:187-195)
 * implemented by
 *   mpmc::flash::Pr76PtFlashBackend
 *     (modules/flash/include/mpmc/flash/pr76_pt_flash_backend.hpp:177-282),
 * one request (= one cell) at a time.  The entry points below take a whole
 * batch of cells of one mixture in structure-of-arrays form, solve them on one
 * GPU, and return the per-cell phase-set status, phase fractions, compositions,
 * ln K, ln phi, Z and, optionally, the implicit sensitivities of
 *   mpmc::flash::differentiate_pr76_pt_vle
 *     (modules/flash/include/mpmc/flash/pr76_sensitivity.hpp:51-390)
 * plus the closure linearisation of
 *   mpmc::physics::build_pr76_pt_vle_closure
 *     (modules/physics/include/mpmc/physics/pr76_thermodynamic_closure.hpp:148-381).
 * The C++ adapter mpmc_hnu_gb300/cpp/gpu_pr76_pt_flash_backend.hpp wraps this
 * ABI behind the reference's PtFlashBackend interface.
 *
 * Conventions
 *  - No exceptions cross this boundary; every function returns an
 *    mpmc_status (0 = success).  mpmc_gpu_flash_last_error() describes the
 *    most recent failure of the calling thread.
 *  - Arrays are structure-of-arrays with the cell index fastest:
 *    element k of cell c lives at a[k * n_cells + c].  Compositions have
 *    k = component; Jacobians have k = row * columns + column.
 *  - Every output pointer may be NULL (that output is skipped).
 *  - Numerical failure of a cell is never an error of the call: it is that
 *    cell's status (MPMC_FLASH_INDETERMINATE), exactly as the reference
 *    publishes PtPhaseSetStatus::indeterminate.
 *  - A handle owns device copies of one mixture's PR76 parameters and is not
 *    reentrant: concurrent calls on one handle must be serialised by the
 *    caller, as for the reference evaluators (pr76_split.hpp:16-18).
 */
#ifndef MPMC_GB300_FLASH_H
#define MPMC_GB300_FLASH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MPMC_GB300_FLASH_ABI_VERSION 1
#define MPMC_MAX_COMPONENTS 20

/* Return codes of the ABI functions. */
typedef enum mpmc_status {
    MPMC_OK = 0,
    MPMC_ERR_INVALID_ARGUMENT = 1, /* reference: std::invalid_argument / length_error */
    MPMC_ERR_DOMAIN = 2,           /* reference: std::domain_error (bad mixture data) */
    MPMC_ERR_CUDA = 3,             /* a CUDA runtime call failed */
    MPMC_ERR_UNSUPPORTED = 4,      /* component count or option outside this library */
    MPMC_ERR_TIMEOUT = 5,          /* a bounded device wait gave up */
    MPMC_ERR_BUSY = 6,             /* flash server: the concurrency limit is reached (the
                                      reference adapter's RESOURCE_EXHAUSTED) */
    MPMC_ERR_DEADLINE = 7          /* flash server: the request's deadline passed before its
                                      results were published (DEADLINE_EXCEEDED) */
} mpmc_status;

/* Per-cell phase-set status, mirroring PtSplitStatus
 * (modules/flash/include/mpmc/flash/pt_split.hpp:71-74). */
enum {
    MPMC_FLASH_SINGLE_PHASE = 0,    /* single_phase_no_instability_found: accepted, 1 phase */
    MPMC_FLASH_TWO_PHASE = 1,       /* two_phase_no_instability_found:   accepted, 2 phases */
    MPMC_FLASH_PHASE_SET_UNSTABLE = 2, /* final common-tangent review found a lower-Gibbs trial */
    MPMC_FLASH_INDETERMINATE = 3,   /* finite search did not settle the phase set */
    MPMC_FLASH_THREE_PHASE = 4,     /* accepted three-phase set (max-3-phase entry points only) */
    MPMC_FLASH_INVALID_REQUEST = -1 /* p, T or feed violate the request contract */
};

/* Outcome of the max-3-phase orchestration per cell, mirroring
 * Pr76PtMax3Status (modules/flash/include/mpmc/flash/pr76_three_phase.hpp:128-135). */
enum {
    MPMC_MAX3_SINGLE_PHASE = 0,
    MPMC_MAX3_TWO_PHASE = 1,             /* the two-phase answer, or a fresh two-phase neighbor */
    MPMC_MAX3_THREE_PHASE = 2,
    MPMC_MAX3_BOUNDARY_UNRESOLVED = 3,   /* a phase disappeared and no neighbor closed */
    MPMC_MAX3_HIGHER_PHASE_COUNT = 4,    /* a three-phase candidate failed its final review */
    MPMC_MAX3_INDETERMINATE = 5
};

/* Algorithm forms (same fixed points, different execution). */
enum {
    MPMC_FORM_PLAIN_FP64 = 0, /* one thread per cell, reference algorithm in FP64 */
    MPMC_FORM_BATCHED = 1,    /* work-queue form, every trial and split attempt an exact FP64 lane-group item */
    MPMC_FORM_MIXED = 2       /* work queue, FP32 bulk iterations + FP64 polish/decisions */
};

/* Work counters per cell (int32 rows of the counters array).  In the mixed
 * form rows 0-2 count FP32 property evaluations and row 5 counts every FP64
 * property evaluation (the cubic is solved by Newton there). */
enum {
    MPMC_COUNTER_INIT_EVALS = 0,   /* property evaluations, initial stability */
    MPMC_COUNTER_SPLIT_EVALS = 1,  /* property evaluations, split attempts */
    MPMC_COUNTER_FINAL_EVALS = 2,  /* property evaluations, final phase-set review */
    MPMC_COUNTER_SPLIT_ITERS = 3,  /* accepted split iterations */
    MPMC_COUNTER_RR_ITERS = 4,     /* Rachford-Rice iterations */
    MPMC_COUNTER_ROOT_ITERS = 5,   /* cubic root iterations */
    MPMC_COUNTER_ATTEMPTS = 6,     /* split attempts */
    MPMC_COUNTER_TRIAL_ITERS = 7,  /* accepted TPD descent iterations */
    MPMC_COUNTER_COUNT = 8
};

/* One mixture: PR76 pure-component data in component order and the
 * row-major symmetric kij matrix (zero diagonal).  Mirrors the numeric
 * content of mpmc::thermodynamics::PrParameterSet
 * (modules/thermodynamics/include/mpmc/thermodynamics/pr_parameters.hpp:46-199). */
typedef struct mpmc_pr76_mixture {
    int32_t n_components;
    const double* critical_temperature_k; /* [n] */
    const double* critical_pressure_pa;   /* [n] */
    const double* acentric_factor;        /* [n] */
    const double* kij;                    /* [n*n] */
} mpmc_pr76_mixture;

/* Option flags (mpmc_flash_options.flags). */
#define MPMC_FLAG_STAGE_TIMING 1 /* record CUDA events around every device stage */
#define MPMC_FLAG_CUDA_GRAPH 2   /* replay solves as CUDA graphs (see mpmc_gpu_flash_solve_device) */
/* Take the sensitivities with the lane-group kernel (component i of a cell on
 * lane i of a group of lanes; rows of the Jacobians and of dF/d ln K in the
 * group's shared memory) instead of one thread per cell.  Same outputs and
 * statuses, to rounding.  Opt-in: checked on the CPU under a warp emulation,
 * not yet timed on a GPU. */
#define MPMC_FLAG_SENSITIVITY_LANES 4
/* The max-3-phase continuation (mpmc_gpu_flash_solve_max3, _hinted) solves
 * the cubic and the Rachford-Rice equations by bracketed Newton with the
 * reference's stopping width, as the flash's FP64 items do, instead of the
 * reference's bisection: fewer FP64 instructions per phase evaluation, the
 * same status on every recorded cell (checked on the CPU), phase sets equal
 * to rounding.  Opt-in: not yet timed on a GPU. */
#define MPMC_FLAG_MAX3_NEWTON_ROOTS 8
/* The mixed form's per-thread FP64 polish as a state machine that makes one
 * property evaluation per loop iteration for every thread, whatever step of
 * its cell's polish that is, so that a warp's lanes evaluate together.  The
 * same arithmetic per cell as the default polish: the outputs are the same
 * (checked on the CPU under a launch emulation).  Opt-in: not yet timed on
 * a GPU. */
#define MPMC_FLAG_POLISH_STREAM 16

typedef struct mpmc_flash_options {
    int32_t form;              /* MPMC_FORM_* */
    int32_t want_sensitivity;  /* nonzero: compute the implicit derivatives */
    int32_t device;            /* CUDA device ordinal */
    int32_t flags;             /* MPMC_FLAG_* */
} mpmc_flash_options;

/* Outputs; layout a[k * n_cells + c].  q = n + 1 reduced columns
 * (p, T, z_0 .. z_{n-2}); the full chart of the per-phase ln phi Jacobians
 * has n + 2 columns (p, T, x_0 .. x_{n-1}) and n + 1 rows (Z, ln phi_0..). */
typedef struct mpmc_flash_outputs {
    int32_t* status;          /* [n_cells]  MPMC_FLASH_* */
    double* vapor_fraction;   /* [n_cells]  beta of the two-phase pair, NaN otherwise */
    double* liquid;           /* [n*n_cells] x (single phase: the feed) */
    double* vapor;            /* [n*n_cells] y */
    double* ln_k;             /* [n*n_cells] ln(y/x) */
    double* ln_phi_liquid;    /* [n*n_cells] (single phase: the feed phase) */
    double* ln_phi_vapor;     /* [n*n_cells] */
    double* z_liquid;         /* [n_cells]  (single phase: Z of the feed phase) */
    double* z_vapor;          /* [n_cells] */
    int32_t* counters;        /* [MPMC_COUNTER_COUNT*n_cells] */
    int32_t* sensitivity_status; /* [n_cells] PtSensitivityStatus, 0 = success */
    double* d_ln_k;           /* [n*q*n_cells] */
    double* d_vapor_fraction; /* [q*n_cells] */
    double* d_liquid;         /* [n*q*n_cells] */
    double* d_vapor;          /* [n*q*n_cells] */
    double* d_z_liquid;       /* [q*n_cells] */
    double* d_z_vapor;        /* [q*n_cells] */
    double* d_rho_liquid;     /* [q*n_cells] molar density gradient */
    double* d_rho_vapor;      /* [q*n_cells] */
    double* jac_liquid;       /* [(n+1)*(n+2)*n_cells] d[Z, ln phi]/d[p, T, x] */
    double* jac_vapor;        /* [(n+1)*(n+2)*n_cells] */
} mpmc_flash_outputs;

/* Three-phase outputs of the max-3-phase entry points; layout a[k * n_cells + c],
 * phase q and component i at row q * n + i.  NaN where the cell has no
 * accepted three-phase set. */
typedef struct mpmc_three_phase_outputs {
    int32_t* max3_status;    /* [n_cells] MPMC_MAX3_*, -1 for an invalid request */
    double* phase_fraction;  /* [3*n_cells] */
    double* composition;     /* [3*n*n_cells] */
    double* ln_phi;          /* [3*n*n_cells] */
    double* z_factor;        /* [3*n_cells] */
} mpmc_three_phase_outputs;

typedef struct mpmc_gpu_flash mpmc_gpu_flash;

/* Create a handle for one mixture on options->device.  Replaces constructing
 * Pr76Phase/Pr76VleEvaluator/Pr76PtFlashBackend for a parameter snapshot
 * (pr76_pt_flash_backend.hpp:179-183; pr76_split.hpp:21-23).  Validates the
 * data the way PrParameterSet::create and Pr76Pure do (finite Tc > 0, Pc > 0,
 * finite omega and kij, symmetric kij with zero diagonal). */
int mpmc_gpu_flash_create(const mpmc_pr76_mixture* mixture, const mpmc_flash_options* options,
                          mpmc_gpu_flash** out);

/* Release the handle and its device memory. */
int mpmc_gpu_flash_destroy(mpmc_gpu_flash* handle);

/* Solve n_cells cells from HOST buffers and write HOST outputs; copies in and
 * out inside the call and returns when the results are on the host.  The
 * batched replacement of PtFlashBackend::solve (pt_flash_backend.hpp:193).
 * p [n_cells] Pa, t [n_cells] K, z [n*n_cells] feed mole fractions. */
int mpmc_gpu_flash_solve(mpmc_gpu_flash* handle, int64_t n_cells, const double* p, const double* t,
                         const double* z, const mpmc_flash_outputs* out);

/* Same, with every pointer (inputs and outputs) in DEVICE memory; enqueued
 * on `stream` (a cudaStream_t, NULL = legacy default stream) and returns
 * without synchronising.  Uses per-handle device scratch that it allocates on
 * first use (and grows as needed).  On a handle created with
 * MPMC_FLAG_CUDA_GRAPH (and without stage timing) the first call for a given
 * cell count and set of buffers captures the launch sequence into a CUDA graph
 * and later identical calls replay it (the last 4 such graphs are kept): the
 * form for a time-stepping loop that flashes the same cell arrays every step.
 * A captured graph reads the buffers it was captured with, so their contents
 * may change between calls but not their addresses. */
int mpmc_gpu_flash_solve_device(mpmc_gpu_flash* handle, int64_t n_cells, const double* p, const double* t,
                                const double* z, const mpmc_flash_outputs* out, void* stream);

/* mpmc_gpu_flash_solve / mpmc_gpu_flash_solve_device with ln K warm starts:
 * ln_k_warm [n*n_cells] (same layout as z; host memory for the first call,
 * device memory for the second) holds each cell's ln(y/x) guess, e.g. from
 * the previous time step or continuation step.  A cell whose warm start has a
 * non-finite entry on a component with z > 0, or is all zero, is solved cold.
 * Work-queue forms only (MPMC_FORM_MIXED, MPMC_FORM_BATCHED; the plain form
 * returns MPMC_ERR_UNSUPPORTED).  ln_k_warm = NULL is the cold solve.
 *
 * The reference has no ln K warm start: its solve hints are TPD start
 * compositions (pt_solve_hints.hpp:26-43).  What a warm start does here is
 * run one split attempt from the guess (pt_split.hpp:275-408), with the same
 * iteration, polish and acceptance rules as a cold attempt, and go straight to
 * the final common-tangent review of that pair (pt_split.hpp:490-512).  The
 * initial stability test and the other attempts are skipped.  The cell is
 * settled only when the review accepts the pair as two_phase, after the same
 * Gibbs-energy check against the feed.  Every other cell (a collapsed or
 * non-converged attempt, an unstable or indeterminate review, or a cold cell)
 * then gets the full cold solve, in a second pass of the same launch. A
 * settled cell's answer is the pair that passed the reference's own
 * acceptance and review tests; a cold solve of the cell can differ from it
 * only where the cold attempts would have selected another local minimum.
 * Each stage time from mpmc_gpu_flash_stage_timings covers both passes;
 * mpmc_gpu_flash_batch_stats counts the warm cells and the ones sent on. */
int mpmc_gpu_flash_solve_warm(mpmc_gpu_flash* handle, int64_t n_cells, const double* p, const double* t,
                              const double* z, const double* ln_k_warm, const mpmc_flash_outputs* out);
int mpmc_gpu_flash_solve_device_warm(mpmc_gpu_flash* handle, int64_t n_cells, const double* p, const double* t,
                                     const double* z, const double* ln_k_warm, const mpmc_flash_outputs* out,
                                     void* stream);

/* mpmc_gpu_flash_solve / _solve_device followed by the reference backend's
 * max-3-phase orchestration for the cells whose two-phase answer is
 * MPMC_FLASH_PHASE_SET_UNSTABLE: Pr76PtFlashBackend::solve runs
 * solve_pr76_pt_max3 (pr76_pt_flash_backend.hpp:190-237,
 * pr76_three_phase.hpp:328-561).  Each such cell's negative witnesses of the
 * final review seed three-phase attempts.  An attempt is a generalized
 * Rachford-Rice balance of three phases and a ln K iteration on both
 * ratios.  A converged three-phase set goes through its own common-tangent
 * review.  A phase that disappears triggers a fresh two-phase solve from the
 * two surviving phases.  The published status follows
 * pt_phase_set.hpp:91-150:
 *   three phases accepted     -> MPMC_FLASH_THREE_PHASE, the set in out3;
 *   fresh two-phase neighbor  -> MPMC_FLASH_TWO_PHASE, its pair in `out`;
 *   three-phase review failed -> MPMC_FLASH_PHASE_SET_UNSTABLE, the base pair kept;
 *   otherwise                 -> MPMC_FLASH_INDETERMINATE, no pair.
 * Cells that are not phase_set_unstable keep their two-phase answer, and
 * out3->max3_status records every cell's outcome.  out->status and
 * out->ln_k are required.  The continuation runs in FP64 with the
 * reference's arithmetic, one cell per warp (the line-search trials of its
 * three-phase attempts on the lanes), for every form.  These calls
 * do not use CUDA graphs, and the sensitivities of a handle created with
 * want_sensitivity are taken after the continuation. */
int mpmc_gpu_flash_solve_max3(mpmc_gpu_flash* handle, int64_t n_cells, const double* p, const double* t,
                              const double* z, const mpmc_flash_outputs* out,
                              const mpmc_three_phase_outputs* out3);
int mpmc_gpu_flash_solve_device_max3(mpmc_gpu_flash* handle, int64_t n_cells, const double* p, const double* t,
                                     const double* z, const mpmc_flash_outputs* out,
                                     const mpmc_three_phase_outputs* out3, void* stream);

/* Caller start hints of a max-3-phase solve: the hints the reference's
 * ordered-path continuation passes from one accepted point to the next
 * (modules/flash/include/mpmc/flash/pr76_pt_continuation.hpp:106-146; the
 * Pr76PtFlashBackendOptions initial_starts, final_starts and
 * three_phase_starts of pr76_pt_flash_backend.hpp:26-40).  Per cell, count
 * (0..3) compositions join the feed stability test and the final review as
 * extra starts; where three_phase is nonzero (count must be 3) they also form a
 * three-phase start, with the fractions of phases 1 and 2, whose attempts
 * run before the automatic ones.  A three-phase start outside the simplex or
 * off the feed's support makes the cell MPMC_FLASH_INVALID_REQUEST, as the
 * reference's start check throws. */
typedef struct mpmc_start_hints {
    const int32_t* count;        /* [n_cells] */
    const double* composition;   /* [3 * n * n_cells]: composition k, component i at (k * n + i) * n_cells + c */
    const int32_t* three_phase;  /* [n_cells] or NULL (then fraction is NULL too) */
    const double* fraction;      /* [2 * n_cells]: phase 1 at c, phase 2 at n_cells + c */
} mpmc_start_hints;

/* mpmc_gpu_flash_solve_max3 / _device_max3 with caller start hints.  These
 * run the plain FP64 kernel -- the reference algorithm -- for every form,
 * followed by the max-3-phase continuation with the same hints.  out->status
 * and out->ln_k are required. */
int mpmc_gpu_flash_solve_hinted(mpmc_gpu_flash* handle, int64_t n_cells, const double* p, const double* t,
                                const double* z, const mpmc_start_hints* hints, const mpmc_flash_outputs* out,
                                const mpmc_three_phase_outputs* out3);
int mpmc_gpu_flash_solve_device_hinted(mpmc_gpu_flash* handle, int64_t n_cells, const double* p, const double* t,
                                       const double* z, const mpmc_start_hints* hints,
                                       const mpmc_flash_outputs* out, const mpmc_three_phase_outputs* out3,
                                       void* stream);

/* The general form of solve_pr76_pt_max3's caller inputs
 * (pr76_three_phase.hpp:328-341): initial_starts, final_starts and one
 * three-phase start per cell, each with arrays of its own, and the two
 * options of Pr76PtMax3Options::two_phase a caller sets in the reference's
 * tests (pt_split.hpp:45-50): initial_stability.automatic_starts and
 * max_split_attempts.  Both options also govern the fresh two-phase solve
 * that follows a three-phase phase disappearance (pr76_three_phase.hpp:413-415).
 * Compositions are laid out as in mpmc_start_hints.  A NULL count array means
 * no starts of that class.  A start off the feed's support, and a feed test
 * left with no start at all, make the cell MPMC_FLASH_INVALID_REQUEST (a
 * domain_error / length_error in the reference). */
typedef struct mpmc_start_hints_ex {
    const int32_t* initial_count;           /* [n_cells], 0..3 */
    const double* initial_composition;      /* [3 * n * n_cells] */
    const int32_t* final_count;             /* [n_cells], 0..3 */
    const double* final_composition;        /* [3 * n * n_cells] */
    const int32_t* three_phase;             /* [n_cells] nonzero: one three-phase start (or NULL) */
    const double* three_phase_composition;  /* [3 * n * n_cells] */
    const double* fraction;                 /* [2 * n_cells] phase_fraction_seed of phases 1 and 2 */
    int32_t initial_automatic_starts;       /* 1: the reference default; 0: the supplied starts only */
    int32_t max_split_attempts;             /* the reference default is 16; 0 .. 65536 */
} mpmc_start_hints_ex;

int mpmc_gpu_flash_solve_hinted_ex(mpmc_gpu_flash* handle, int64_t n_cells, const double* p, const double* t,
                                   const double* z, const mpmc_start_hints_ex* hints, const mpmc_flash_outputs* out,
                                   const mpmc_three_phase_outputs* out3);
int mpmc_gpu_flash_solve_device_hinted_ex(mpmc_gpu_flash* handle, int64_t n_cells, const double* p,
                                          const double* t, const double* z, const mpmc_start_hints_ex* hints,
                                          const mpmc_flash_outputs* out, const mpmc_three_phase_outputs* out3,
                                          void* stream);

/* ------------------------------------------------------------------------
 * Selected-phase property chart: the flow module's per-cell property and
 * Jacobian publication on a frozen natural-variable chart,
 *   mpmc::flow::evaluate_pr76_selected_phase_property_chart
 *     (modules/flow/include/mpmc/flow/pr76_selected_phase_property_closure.hpp:533-822)
 * over the fixed-selected-branch closure Pr76SelectedPhasePropertyClosure
 * (:258-475), which the production cell evaluators call once per cell
 * (Pr76ProductionCellEvaluatorTraits::evaluate_property_chart,
 * modules/flow/discretization/petsc/include/mpmc/flow_discretization_petsc/
 * pr76_production_cell_evaluator.hpp:88-101).  Here one call evaluates a
 * whole batch of cells that share the closure (phase count, selected roots,
 * molar masses and transport/caloric model).
 *
 * Chart of a cell with P phases and n components (the layout of
 * NaturalVariableLayoutDescriptor, natural_variable_cell_state.hpp:66-216),
 * q = P n + 1 unknowns:
 *   q[0] = p [Pa], q[1] = T [K], q[2 .. P] = saturations of phases 0..P-2,
 *   then per phase k the n - 1 independent mole fractions in component order
 *   with the phase's dependent (pivot) component left out; the dependent
 *   fraction is 1 - sum of the others.
 * Outputs per cell, rows in this order (P (5 + n) + (P - 1) n rows):
 *   per phase k, at row k (5 + n): molar density [mol/m3], mass density
 *   [kg/m3], dynamic viscosity [Pa s], specific enthalpy [J/kg], specific
 *   internal energy u = h - p / rho_mass [J/kg], ln phi_0 .. ln phi_{n-1};
 *   then per phase k >= 1 and component i the equilibrium residual
 *   ln(x_0,i / x_k,i) + ln phi_0,i - ln phi_k,i.
 * values[row * n_cells + c] holds the value and
 * jacobian[(row * q + column) * n_cells + c] its derivative by chart column.
 *
 * The viscosity and enthalpy are the caller's model in the reference (the
 * closure's TransportCaloricProvider, :258-270).  This library evaluates the
 * affine model
 *   f = c[0] + c[1] p + c[2] T + sum_i c[7+i] x_i + c[3] rho + c[4] M
 *       + c[5] rho_mass + c[6] root_index
 * with M = sum_i x_i M_i, once with the viscosity and once with the enthalpy
 * coefficients (7 + n each).  A nonlinear correlation is not available on the
 * device; such a caller evaluates it from the published density, composition
 * and their Jacobians. */
typedef struct mpmc_property_chart_spec {
    int32_t phase_count;           /* P, 1..3 */
    int32_t root_index[3];         /* Pr76SelectedPhase::root_index of phase 0..P-1: the
                                      index into the PR76 roots ordered by increasing Z */
    const double* molar_mass;      /* [n] kg/mol, finite and > 0 */
    const double* viscosity;       /* [7 + n] affine coefficients */
    const double* enthalpy;        /* [7 + n] affine coefficients */
} mpmc_property_chart_spec;

/* Per-cell status of the chart.  The reference throws; the class of each
 * throw is kept so the production evaluator's mapping (domain errors ->
 * NaturalVariableSnesEvaluationStatus3D::domain_error, std::out_of_range ->
 * PETSC_ERR_PLIB, pr76_production_cell_evaluator.hpp:42-86) applies. */
typedef enum mpmc_chart_status {
    MPMC_CHART_OK = 0,
    MPMC_CHART_INPUT_DOMAIN = 1,     /* non-finite chart entry; p, T, a mole fraction or
                                        M not finite and positive (range/domain_error) */
    MPMC_CHART_EOS_DOMAIN = 2,       /* the EOS rejected the state: A, B, ln phi or Z not
                                        representable (range/domain_error) */
    MPMC_CHART_ROOT_UNRESOLVED = 3,  /* Pr76PhaseError: near-multiple, iteration limit or
                                        unrepresentable root set */
    MPMC_CHART_ROOT_INDEX = 4,       /* std::out_of_range: the selected root does not exist */
    MPMC_CHART_ILL_CONDITIONED = 5,  /* Pr76PhaseError: selected root without a reliable
                                        derivative */
    MPMC_CHART_PROPERTY_DOMAIN = 6   /* density, mass density or viscosity not positive, or
                                        a non-finite property or derivative (range/domain_error) */
} mpmc_chart_status;

typedef struct mpmc_property_chart_outputs {
    int32_t* status;   /* [n_cells] mpmc_chart_status */
    double* values;    /* [rows * n_cells]; NaN rows for a failed cell */
    double* jacobian;  /* [rows * q * n_cells]; NaN for a failed cell */
} mpmc_property_chart_outputs;

/* Property chart of n_cells cells: q [(P n + 1) * n_cells] chart values;
 * dependent [P * n_cells] the dependent component of phase k of cell c at
 * dependent[k * n_cells + c], or NULL for the last component everywhere
 * (NaturalVariableCompositionPivot3P::fixed_last).  Host buffers: the call
 * copies, evaluates and copies back before returning.  One thread per cell in
 * FP64; the Jacobian is the closed form of the reference's forward-AD
 * quantity. */
int mpmc_gpu_flash_property_chart(mpmc_gpu_flash* handle, int64_t n_cells, const mpmc_property_chart_spec* spec,
                                  const double* q, const int32_t* dependent,
                                  const mpmc_property_chart_outputs* out);
/* The same on device buffers, enqueued on `stream` (NULL = default stream);
 * returns without synchronising. */
int mpmc_gpu_flash_property_chart_device(mpmc_gpu_flash* handle, int64_t n_cells,
                                         const mpmc_property_chart_spec* spec, const double* q,
                                         const int32_t* dependent, const mpmc_property_chart_outputs* out,
                                         void* stream);

/* Largest device scratch, in bytes, of mpmc_gpu_flash_solve_device_noalloc:
 * a fixed 48 MiB array in the library's device code. */
#define MPMC_NOALLOC_SCRATCH_BYTES (48u << 20)

/* mpmc_gpu_flash_solve_device for callers that must not allocate device memory
 * during a solve: code that runs while a CUDA graph is being captured on its
 * stream, a solver callback inside a host application whose memory pool owns
 * every allocation, or a latency-bound request loop that cannot afford an
 * allocation on its path.  No counterpart in the reference (whose backend
 * allocates host vectors per solve, pt_flash_backend.hpp:125-182).
 *
 * Mixed-precision handles only (MPMC_FORM_MIXED; other forms return
 * MPMC_ERR_UNSUPPORTED).  The work buffers of the solve live in one fixed
 * MPMC_NOALLOC_SCRATCH_BYTES array of device memory per device; a batch whose
 * buffers do not fit (about 2,700 cells at 20 components, 7,300 at 10, more
 * with fewer components) returns MPMC_ERR_INVALID_ARGUMENT with the size in
 * the message.  The queue of FP64 attempt continuations takes the rest of the
 * array, up to one entry per attempt (16 per cell): in a batch of hard cells
 * whose queue still overflows, the cells that do not fit run the plain FP64
 * fallback -- the same answers, slower.  The first call on a device looks the array's address up
 * (cudaGetSymbolAddress, with that device current), and the first launch of
 * each of its kernels in the process lets the CUDA driver size the context's
 * local-memory (stack) reservation for that kernel -- the implicit-sensitivity
 * kernel has the largest frame, so with want_sensitivity the first call may
 * grow that reservation.  Make one call of each kind (with and without
 * sensitivities, at each component count used) before any stream capture
 * and before entering code that must not allocate.  After that the call
 * allocates nothing: it validates,
 * enqueues its kernels and a zeroing of the work counters on `stream`, and
 * returns without synchronising.  All handles on a device share the array, so
 * calls whose work overlaps on the device (two streams, or two host threads)
 * race and corrupt each other: serialise them, e.g. on one stream.  When the
 * handle was created with want_sensitivity, the flash fields the sensitivity
 * kernel reads back (status, vapor_fraction, liquid, vapor, ln_k, z_liquid,
 * z_vapor) must be provided, because there is no scratch to route them to.
 * Stage timing is not recorded.  Results equal those of
 * mpmc_gpu_flash_solve_device on the same inputs. */
int mpmc_gpu_flash_solve_device_noalloc(mpmc_gpu_flash* handle, int64_t n_cells, const double* p,
                                        const double* t, const double* z, const mpmc_flash_outputs* out,
                                        void* stream);

/* Launch shape of the mixed form on this handle, as chosen by an autotuner
 * (mpmc_hnu_gb300/autotune.py) or by hand; count values, the rest default.
 *   [0] FP32 trial blocks per SM        [1] FP32 attempt blocks per SM
 *   [2] FP64 trial-item blocks per SM   [3] FP64 attempt and polish blocks per SM
 *   [4] per-cell kernel blocks per SM   [5] item form: bit 0 feed trials, bit 1
 *       review trials, bit 2 attempts run one item per thread instead of one
 *       per lane group; the polish runs one cell per thread with bit 3, one per
 *       lane group with bit 4 (default: per thread up to 12 components);
 *       FP64 trial items run 32 / S to a warp (S = the component capacity
 *       rounded to a power of two), or one per warp with bit 5; FP64
 *       attempt items one per warp with bit 6, 32 / S to a warp with bit 7
 *       (default: packed up to 8 components)
 *   [6] successive-substitution -> Newton switch: the FP32 |r| (in units of
 *       1e-6) at which the FP32 ln K iteration hands over to the FP64 polish
 *   [7] cell ranges (1-8) a solve is split into, each a solve of its own on
 *       its own stream, so that the long last items of one range overlap the
 *       bulk stages of the others (default 1; every range keeps at least
 *       65,536 cells; the outputs do not depend on it)
 *   [8] FP32 trial screen: a stability trial whose FP32 descent projects
 *       more FP64 iterations than this (1-512) is re-run exactly in FP64
 *       instead of being decided from its FP32 end point
 *   [9] an undecided trial or unsettled split attempt whose FP32 run took at
 *       least this many iterations (1-512) runs from its start in FP64
 *       instead of continuing from its FP32 end point
 * 0 selects the default (occupancy-derived residency, lane-group items,
 * switch at 2e-5).  Results do not depend on the shape beyond the rounding of
 * where each iteration stops.  Drops the handle's captured graphs.  No
 * counterpart in the reference. */
int mpmc_gpu_flash_set_launch_shape(mpmc_gpu_flash* handle, const int32_t* values, int count);

/* Device time in milliseconds of every stage of the last solve on a handle
 * created with MPMC_FLAG_STAGE_TIMING (waits for that solve to finish).
 * Stages, in order -- plain form: flash, sensitivity; mixed form: setup,
 * feed_trials, feed_classify, feed_trials64, decide, split, polish, open32, compete, split64,
 * select64, relist, review_trials, review_classify, review_trials64, finish,
 * fallback, sensitivity.  Writes up to `capacity` values and returns the
 * number of stages (0 if timing is off or nothing ran).  Diagnostic entry
 * point with no counterpart in the reference (whose solver results carry
 * work counters only, pt_stability.hpp:66-76). */
int mpmc_gpu_flash_stage_timings(mpmc_gpu_flash* handle, float* ms, int capacity);

/* Work statistics of the last work-queue solve on a handle (waits for the
 * device): [0] feed trials continued in FP64 from their FP32 end point,
 * [1] feed trials re-run exactly in FP64, [2] review trials continued,
 * [3] review trials re-run, [4] cells sent to the plain FP64 fallback
 * (nonsmooth feed phase), [5..7] cells whose split attempts were continued in
 * FP64 because no FP32 attempt settled / the polish did not converge / the
 * polished pair failed the acceptance rules, [8] cells with unusable
 * constants, [9] cells whose two best attempts were both polished,
 * [10] FP64 trial items, [11] FP64 attempt items, [12] cells polished,
 * [13] cells whose attempts were selected in FP64, [14] slow FP32 trials
 * whose exact re-run was skipped because another trial of the same test was
 * already negative, [15] split attempts classified as ending at the
 * iteration limit without an FP64 run, [16] cells run from their ln K warm
 * start, [17] of those, cells whose pair was not accepted and that took the
 * cold pass, [18] of those, cells with no converged attempt, [19] of those,
 * cells whose review found a negative TPD, [20] cells whose polished pair
 * waited on attempts that FP32 left open, [21] of those, cells where some open
 * attempt could still change the selection and was continued in FP64, [22]
 * cells whose polished attempt the linear replay of the reference's line
 * search showed stalling or near the iteration limit, so every attempt of the
 * cell was continued in FP64 instead (every entry summed over the solve's
 * cell ranges); [23]-[27] FP64 property evaluations
 * of the feed phase (setup), the FP64 feed-test trial items, the FP64 review
 * trial items, the Newton polish and the FP64 attempt continuations; [28]
 * closed-form Jacobians the polish factorised and [29] its chord-step solves
 * (the algorithmic work of each FP64 stage); [30] cells the plain FP64
 * fallback solved (a nonsmooth feed phase, unusable constants, or FP64
 * attempt items beyond the queue's capacity); [31] cells the exact sub-solve
 * solved again with every trial and attempt in FP64 (no FP32 attempt
 * converged, or the replay put the polished attempt at risk; the
 * sub-solve's own work is not in [0]-[29]).  After a warm-start solve, [0]-[15] and [30] count the last pass and [20]-[29] and
 * [31] every pass.
 * Writes up to `capacity` values; returns the number available (0 for the
 * plain form).  Diagnostic entry point with no counterpart in the reference. */
int mpmc_gpu_flash_batch_stats(mpmc_gpu_flash* handle, int64_t* out, int capacity);

/* Number of components of the handle's mixture. */
int mpmc_gpu_flash_components(const mpmc_gpu_flash* handle);

/* Thread-local description of the last failure ("" if none). */
const char* mpmc_gpu_flash_last_error(void);

/* ABI version (MPMC_GB300_FLASH_ABI_VERSION). */
int mpmc_gpu_flash_abi_version(void);

/* ------------------------------------------------------------------------
 * Flash server: the PT service path as a device-resident request loop
 * (replaces the per-request PtService::solve -> PtFlashBackend::solve calls,
 * pt_service.hpp:335-369, for many concurrent clients).
 *
 * Requests (one mixture, any cell count up to max_batch_cells) are queued by
 * mpmc_flash_server_submit from any thread and return a ticket at once.  A
 * worker thread keeps `slots` device batches in flight, each on its own CUDA
 * stream with its own device buffers: whenever a slot is free it takes the
 * oldest waiting request and every other waiting request of the same mixture
 * that still fits, copies them in, launches the flash and copies the results
 * out, so requests that arrive while others run are admitted as slots free up
 * and their work overlaps on the device (continuous batching).  Each mixture's
 * prepared constants stay on the device from add_mixture to destroy.  Slots
 * are admitted by memory: the server holds at most memory_budget_bytes of
 * device memory and creates only as many slots as fit.  Results are per cell
 * and independent of what else is in the batch: a request's outputs are the
 * same alone and in any mix.  Flash fields only (status .. counters); the
 * sensitivity fields of `out` must be NULL.  Without MPMC_SERVER_WARM_CACHE
 * results equal those of mpmc_gpu_flash_solve.
 *
 * MPMC_SERVER_WARM_CACHE (mixed form): each mixture also keeps, on the device,
 * the ln K of its recently solved two-phase cells, keyed by the composition
 * (65,536 entries per mixture, a newer cell overwriting an older one in the
 * same entry).  A cell of a later request with a cached composition, p within
 * a factor exp(0.25) and T within 15 K starts from that ln K, as
 * mpmc_gpu_flash_solve_warm does (one attempt from the start and the
 * reference's final review; anything else takes the full cold solve).  A
 * request's statuses then equal the cold solve's and its pairs agree with it
 * to the polish tolerance, but its raw values depend on what was solved
 * before.  The reference re-solves every request cold; its solve hints are
 * TPD start compositions (pt_solve_hints.hpp:26-43). */
#define MPMC_SERVER_WARM_CACHE 1

typedef struct mpmc_server_options {
    int32_t device;
    int32_t slots;                /* batches in flight; 0 = 4 */
    int64_t max_batch_cells;      /* cells per device batch (and per request); 0 = 65536 */
    int64_t memory_budget_bytes;  /* device memory the server may hold; 0 = 40 GiB */
    int32_t form;                 /* MPMC_FORM_MIXED or MPMC_FORM_PLAIN_FP64 (= 0): set it explicitly */
    int32_t flags;                /* MPMC_SERVER_WARM_CACHE or 0 */
} mpmc_server_options;

/* Scheduling and admission policy of a server (mpmc_flash_server_set_policy,
 * before the first submit; every field 0 = the default in brackets).
 *  - small_request_cells: requests of at most this many cells are latency
 *    requests [0: none].  The first `latency_slots` slots [0] serve only them,
 *    on streams of the highest priority, in batches of at most
 *    latency_batch_cells cells [max_batch_cells]; the other slots take them
 *    only when no larger work waits.
 *  - chunk_cells: a request is solved in tasks of at most this many cells
 *    [max_batch_cells], so a large request's launches stay short and
 *    interleave with others; max_request_cells [max_batch_cells] bounds a
 *    request (at most 4096 chunks).
 *  - max_in_flight: submitted and not yet completed requests [0: no limit];
 *    a submit beyond it fails at once with MPMC_ERR_BUSY, as the reference
 *    adapter refuses a solve beyond max_concurrent_solves
 *    (pt_grpc_adapter.cpp:547-558, 622-626).
 *  - max_deadline_us: the largest deadline mpmc_flash_server_submit_deadline
 *    accepts [0: any], as the adapter's max_solve_deadline
 *    (pt_grpc_adapter.cpp:377-396). */
typedef struct mpmc_server_policy {
    int64_t small_request_cells;
    int32_t latency_slots;
    int32_t pad;
    int64_t latency_batch_cells;
    int64_t chunk_cells;
    int64_t max_request_cells;
    int64_t max_in_flight;
    int64_t max_deadline_us;
} mpmc_server_policy;

typedef struct mpmc_flash_server mpmc_flash_server;

int mpmc_flash_server_create(const mpmc_server_options* options, mpmc_flash_server** out);

/* Set the scheduling and admission policy (see mpmc_server_policy); before
 * the first submit.  No counterpart in the reference beyond the limits cited
 * there. */
int mpmc_flash_server_set_policy(mpmc_flash_server* server, const mpmc_server_policy* policy);

/* Register a mixture (validated like mpmc_gpu_flash_create); its id is used
 * by submit.  Up to 64 mixtures per server. */
int mpmc_flash_server_add_mixture(mpmc_flash_server* server, const mpmc_pr76_mixture* mixture,
                                  int32_t* mixture_id);

/* Queue one request.  p, t, z and the output buffers are host memory owned by
 * the caller and must stay valid until mpmc_flash_server_wait returns for the
 * ticket; layouts as in mpmc_gpu_flash_solve for n_cells cells. */
int mpmc_flash_server_submit(mpmc_flash_server* server, int32_t mixture_id, int64_t n_cells, const double* p,
                             const double* t, const double* z, const mpmc_flash_outputs* out, uint64_t* ticket);

/* mpmc_flash_server_submit with a deadline deadline_us > 0 microseconds after
 * the call, as the reference adapter requires a finite RPC deadline
 * (pt_grpc_adapter.cpp:377-396): a request whose deadline passes before its
 * tasks are launched is dropped, and one whose deadline passes before its
 * results are published gets none; mpmc_flash_server_wait then returns
 * MPMC_ERR_DEADLINE and the request's outputs are not written (rows of a task
 * already scattered stay).  A deadline above the policy's max_deadline_us is
 * MPMC_ERR_INVALID_ARGUMENT. */
int mpmc_flash_server_submit_deadline(mpmc_flash_server* server, int32_t mixture_id, int64_t n_cells,
                                      const double* p, const double* t, const double* z,
                                      const mpmc_flash_outputs* out, int64_t deadline_us, uint64_t* ticket);

/* Wait for a ticket (timeout_us < 0: no limit).  On return 0 the outputs are
 * written and *latency_s (optional) is the time from submit to completion.
 * MPMC_ERR_TIMEOUT if the time ran out; the request stays queued. */
int mpmc_flash_server_wait(mpmc_flash_server* server, uint64_t ticket, int64_t timeout_us, double* latency_s);

/* Counters: [0] submitted, [1] completed, [2] device batches, [3] cells,
 * [4] slots, [5] device bytes per slot, [6] most requests in one batch,
 * [7] most slots busy at once, [8] submits refused by max_in_flight,
 * [9] requests whose deadline passed, [10] requests in flight, [11] cells
 * started from the warm-start cache.  Returns the number written. */
int mpmc_flash_server_stats(mpmc_flash_server* server, int64_t* out, int capacity);

/* Finish the queued requests, stop the worker and free everything. */
int mpmc_flash_server_destroy(mpmc_flash_server* server);

#ifdef __cplusplus
}
#endif
#endif /* MPMC_GB300_FLASH_H */
