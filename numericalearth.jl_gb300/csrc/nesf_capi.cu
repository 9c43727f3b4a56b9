// nesf_capi.cu -- the extern "C" entry points of libnesf.so (declared in include/nesf.h).
//
// Validation, parameter conversion and dispatch to the kernels. Each entry point
// returns an nesf_status and records a message for nesf_last_error() on failure.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <cstdarg>
#include <mutex>
#include <string>
#include <vector>
#include <new>

#include "nesf_solve.cuh"
#include "nesf_exchange.cuh"

using namespace nesf;

struct nesf_context {
    int device;
    DevStats* d_stats;          // device statistics accumulator
    DevStats* h_stats;          // pinned host copy
    DevIface<double>* d_p64;    // per-member parameters (ensemble)
    DevIface<float>* d_p32;
    int32_t capacity_members;
    uint32_t* d_replay;         // the deferred-cell queues of the FP32 solvers (4 parts x capacity)
    float* d_pstate;            // pass 1's state of the polish queue's entries (sea-ice solves)
    int64_t pstate_capacity;
    unsigned int* d_replay_count;   // [8]: the queue parts [0..3], pass 1's fetch counter [4]
    int64_t replay_capacity;
    uint32_t* d_work;           // compacted work lists of the solves
    unsigned int* d_work_count; // two counters per ensemble member
    int64_t work_capacity;
    int32_t work_members;
    void* d_partials;           // per-block partial sums of the area integrals
    float* d_feat;              // warm start: features (8 floats) and guesses (4) per work-list slot
    float* d_guess;
    int64_t warm_capacity;
    float* d_anchor;            // the adaptive pass 1's cancelling differences per work-list slot
    int64_t anchor_capacity;
    // the coupling step's second lane: scratch of the sea-ice solve, its stream, fork/join events
    nesf_context* aux;
    cudaStream_t side;
    cudaEvent_t ev_fork, ev_ice, ev_join, ev_ocean;
    // the sea-ice solve's replay stream beside its polish pass, with fork/join events, and its
    // early lane (the calm cells' replays beside pass 1)
    cudaStream_t tail;
    cudaEvent_t ev_tail_fork, ev_tail_join;
    cudaStream_t early;
    cudaEvent_t ev_early_fork, ev_early_join;
    nesf_tuning tuning;         // launch shapes and schedule (nesf_set_tuning, nesf_autotune)
    struct TraceBuf* trace;     // kernel-boundary trace (nesf_trace_enable); the lane context borrows it
    bool trace_owned;
    std::mutex lock;            // serialises use of the scratch above
};

// The events of a trace and the tracer hook the launchers call.
struct TraceBuf {
    bool on;
    int n;
    cudaEvent_t ev[NESF_TRACE_MAX];
    const char* name[NESF_TRACE_MAX];
    cudaStream_t stream[NESF_TRACE_MAX];
    Tracer hook;
};

static void trace_record(void* self, const char* name, cudaStream_t s) {
    TraceBuf* t = (TraceBuf*)self;
    if (!t->on || t->n >= NESF_TRACE_MAX) return;
    // under stream capture the record becomes an event-record node of the graph
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) return;
    unsigned flags = cap == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault;
    if (cudaEventRecordWithFlags(t->ev[t->n], s, flags) != cudaSuccess) return;
    t->name[t->n] = name;
    t->stream[t->n] = s;
    t->n++;
}

static const Tracer* tracer_of(const nesf_context* ctx) {
    return ctx && ctx->trace && ctx->trace->on ? &ctx->trace->hook : nullptr;
}

// The defaults of nesf_tuning's fields.
static nesf_tuning default_tuning() {
    nesf_tuning t{};
    t.solve_block = 128;
    t.deferred_per_sm = 4;
    t.infer_per_sm = 4;
    t.two_lanes = 1;
    t.io_overlap = 1;
    t.pass1_fetch = 2;
    t.refill_lanes = 8;
    t.early_ocean_classify = 0;
    t.ice_deferred_per_sm = 0;
    t.cells_per_thread = 1;
    return t;
}

namespace nesf {
cudaError_t launch_integrals(const nesf_integral_fields& f, void* partials, int max_blocks, double* result,
                             cudaStream_t s);
}
// blocks of the area-integral pass (x 16 integrals x 16 B of partial sums: 256 KiB)
static const int kIntegralBlocks = 1024;

static thread_local char g_err[512] = "";

static int fail(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    return code;
}

static int cuda_fail(cudaError_t e, const char* what) {
    return fail(NESF_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define NESF_CUDA(call)                                   \
    do {                                                  \
        cudaError_t e_ = (call);                          \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

// Switches to the context's device for the duration of a call.
struct DeviceGuard {
    int prev = -1;
    bool ok = true;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) { ok = false; return; }
        if (prev != dev && cudaSetDevice(dev) != cudaSuccess) ok = false;
    }
    ~DeviceGuard() {
        int cur;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

extern "C" {

int32_t nesf_abi_version(void) { return NESF_ABI_VERSION; }
const char* nesf_version(void) { return "nesf 0.1.0 (sm_103a)"; }
const char* nesf_last_error(void) { return g_err; }

int32_t nesf_struct_sizes(int64_t* sizes, int32_t n) {
    const int64_t s[] = {
        (int64_t)sizeof(nesf_grid), (int64_t)sizeof(nesf_thermodynamics_parameters),
        (int64_t)sizeof(nesf_stability_function), (int64_t)sizeof(nesf_roughness_length),
        (int64_t)sizeof(nesf_similarity_theory_fluxes), (int64_t)sizeof(nesf_interface_params),
        (int64_t)sizeof(nesf_solver_options), (int64_t)sizeof(nesf_stats), (int64_t)sizeof(nesf_ao_fields),
        (int64_t)sizeof(nesf_ai_fields), (int64_t)sizeof(nesf_io_params), (int64_t)sizeof(nesf_io_fields),
        (int64_t)sizeof(nesf_atmos_grid), (int64_t)sizeof(nesf_exchange_coords), (int64_t)sizeof(nesf_interp_fields),
        (int64_t)sizeof(nesf_assembly_params), (int64_t)sizeof(nesf_assembly_fields),
        (int64_t)sizeof(nesf_coupling_step_args), (int64_t)sizeof(nesf_integral_fields),
        (int64_t)sizeof(nesf_tuning), (int64_t)sizeof(nesf_trace_entry), (int64_t)sizeof(nesf_coefficient_fluxes),
        (int64_t)sizeof(nesf_al_fields), (int64_t)sizeof(nesf_land_radiation_params),
        (int64_t)sizeof(nesf_land_flux_fields), (int64_t)sizeof(nesf_tuning_key)};
    int32_t m = (int32_t)(sizeof s / sizeof s[0]);
    for (int32_t k = 0; k < n && k < m; k++) sizes[k] = s[k];
    return m;
}

// ---------------------------------------------------------------- defaults
void nesf_default_thermodynamics(nesf_thermodynamics_parameters* t) {
    // src/Atmospheres/thermodynamic_parameters.jl:61-69,106-116,149-165
    t->gas_constant = 8.3144598;
    t->dry_air_molar_mass = 0.02897;
    t->water_molar_mass = 0.018015;
    t->dry_air_adiabatic_exponent = 2.0 / 7.0;
    t->water_vapor_heat_capacity = 1859;
    t->liquid_water_heat_capacity = 4181;
    t->water_ice_heat_capacity = 2100;
    t->reference_vaporization_enthalpy = 2500800;
    t->reference_sublimation_enthalpy = 2834400;
    t->reference_temperature = 273.16;
    t->triple_point_temperature = 273.16;
    t->triple_point_pressure = 611.657;
}

static void default_fluxes(nesf_similarity_theory_fluxes* f, bool ice) {
    memset(f, 0, sizeof *f);
    // similarity_theory_turbulent_fluxes.jl:174-214
    f->von_karman_constant = 0.4;
    f->turbulent_prandtl_number = 1;
    f->subgrid_kind = NESF_SUBGRID_CONVECTIVE;
    f->gustiness_parameter = 1.2;
    f->minimum_gustiness = 0.01;
    f->similarity_form = NESF_PROFILE_LOGARITHMIC;
    const double pi = 3.14159265358979323846;
    if (!ice) {
        // Edson et al. 2013 (:487-499, :571-584)
        double m[11] = {50.0, 0.35, 0.7, 0.75, 5 / 0.35, 15.0, 2.0, pi / 2, 10.15, 3.0, pi / sqrt(3.0)};
        double s[12] = {50.0, 0.35, 2.0 / 3.0, 3.0 / 2.0, 14.28, 8.525, 15.0, 2.0, 0.0, 34.15, 3.0, pi / sqrt(3.0)};
        f->stability[0].kind = NESF_PSI_EDSON_MOMENTUM;
        for (int k = 0; k < 11; k++) f->stability[0].c[k] = m[k];
        for (int n = 1; n < 3; n++) {
            f->stability[n].kind = NESF_PSI_EDSON_SCALAR;
            for (int k = 0; k < 12; k++) f->stability[n].c[k] = s[k];
        }
    } else {
        // Paulson unstable + SHEBA stable (:637-640, 659-663, 683-703, 779-789)
        f->stability[0].kind = NESF_PSI_SHEBA_PAULSON_MOMENTUM;
        f->stability[0].c[0] = 6.5; f->stability[0].c[1] = 1.3;
        f->stability[0].c[2] = 16.0; f->stability[0].c[3] = pi / 2;
        for (int n = 1; n < 3; n++) {
            f->stability[n].kind = NESF_PSI_SHEBA_PAULSON_SCALAR;
            f->stability[n].c[0] = 5.0; f->stability[n].c[1] = 5.0; f->stability[n].c[2] = 3.0;
            f->stability[n].c[3] = 16.0;
        }
    }
    // roughness_lengths.jl:93-139
    nesf_roughness_length* r = &f->roughness[0];
    r->kind = NESF_ROUGHNESS_MOMENTUM;
    r->gravitational_acceleration = 9.80665;
    r->air_kinematic_viscosity = 1.5e-5;
    r->charnock = 0.02;
    r->smooth_wall_parameter = 0.11;
    r->maximum_roughness_length = 1.0;
    for (int n = 1; n < 3; n++) {
        nesf_roughness_length* q = &f->roughness[n];
        q->kind = NESF_ROUGHNESS_SCALAR;
        q->air_kinematic_viscosity = 1.5e-5;
        q->reynolds_A = 5.85e-5;
        q->reynolds_b = 0.72;
        q->maximum_roughness_length = 1.6e-4;
    }
    f->stop_kind = NESF_STOP_CONVERGENCE;
    f->maxiter = 100;
    f->tolerance = 1e-8;
}

void nesf_default_ao_params(nesf_interface_params* p) {
    memset(p, 0, sizeof *p);
    default_fluxes(&p->fluxes, false);
    nesf_default_thermodynamics(&p->thermo);
    p->humidity_phase = NESF_PHASE_LIQUID;       // component_interfaces.jl:353-358
    p->has_water_mole_fraction = 1;
    p->water_mole_fraction = 0.98;
    p->velocity_formulation = NESF_RELATIVE_VELOCITY;
    p->temperature_formulation = NESF_BULK_TEMPERATURE;
    p->max_delta_T = 5;
    p->gravitational_acceleration = 9.80665;
    p->surface_layer_height = 10;
    p->boundary_layer_height = 512;
    p->interior_temperature_offset = 273.15;
    p->interface_temperature_offset = 273.15;
    p->stefan_boltzmann_constant = 5.670374419e-8;
    p->albedo = 0;          // radiation off by default (has_radiation = 0)
    p->emissivity = 0;
    p->liquidus_freshwater_melting_temperature = 0;
    p->liquidus_slope = 0.054;
    p->interior_reference_density = 1020;
    p->interior_heat_capacity = 3991.86795711963;
}

void nesf_default_coefficient_fluxes(nesf_coefficient_fluxes* c, int32_t kind) {
    memset(c, 0, sizeof *c);
    c->kind = kind;
    c->stop_kind = NESF_STOP_CONVERGENCE;    // coefficient_based_turbulent_fluxes.jl:215-229
    c->maxiter = 20;
    c->tolerance = 1e-8;
    if (kind == NESF_COEFFICIENTS_CONSTANT) {
        c->momentum = c->temperature = c->water_vapor = 1e-3;   // :216
        return;
    }
    c->von_karman_constant = 0.4;            // :92-99
    c->drag_a = 2.7;                         // :30-37
    c->drag_b = 0.142;
    c->drag_c = 1 / 13.09;
    c->drag_d = 3.14807e-10;
    c->high_wind_speed_threshold = 33;
    c->high_wind_drag_coefficient = 2.34e-3;
    c->minimum_wind_speed = 0.5;
    c->reference_height = 10;
    c->stable_heat_transfer_coefficient = 18;
    c->unstable_heat_transfer_coefficient = 32.7;
    c->moisture_transfer_coefficient = 34.6;
    // large_yeager_stability_functions (similarity_theory_turbulent_fluxes.jl:766-771): linear
    // stable branch (psi = -5 zeta, zeta <= 10; :742-752) + Paulson (:683-710)
    c->stability[0].kind = NESF_PSI_LINEAR_PAULSON_MOMENTUM;
    c->stability[0].c[0] = 5; c->stability[0].c[1] = 10; c->stability[0].c[2] = 16; c->stability[0].c[3] = M_PI / 2;
    c->stability[1].kind = NESF_PSI_LINEAR_PAULSON_SCALAR;
    c->stability[1].c[0] = 5; c->stability[1].c[1] = 10; c->stability[1].c[2] = 16;
}

void nesf_default_al_params(nesf_interface_params* p) {
    nesf_default_ao_params(p);
    // default_atmosphere_land_fluxes (component_interfaces.jl:514-521): SimilarityTheoryFluxes
    // with the Large-Yeager stability functions (atmosphere_land_stability_functions,
    // similarity_theory_turbulent_fluxes.jl:776-777) and constant roughness lengths
    nesf_similarity_theory_fluxes& f = p->fluxes;
    nesf_coefficient_fluxes ly;
    nesf_default_coefficient_fluxes(&ly, NESF_COEFFICIENTS_LARGE_YEAGER);
    f.stability[0] = ly.stability[0];
    f.stability[1] = ly.stability[1];
    f.stability[2] = ly.stability[1];
    const double rough[3] = {0.1, 0.01, 0.01};
    for (int n = 0; n < 3; n++) {
        memset(&f.roughness[n], 0, sizeof f.roughness[n]);
        f.roughness[n].kind = NESF_ROUGHNESS_CONSTANT;
        f.roughness[n].value = rough[n];
    }
    p->humidity_phase = NESF_PHASE_LIQUID;      // BulkHumidity(Liquid) (:501-503)
    p->has_water_mole_fraction = 0;
    p->water_mole_fraction = 1;
    p->humidity_formulation = NESF_HUMIDITY_BULK;
    p->evaporation_efficiency = 1;
    p->interior_temperature_offset = 0;        // land temperatures in kelvin
    p->interface_temperature_offset = 0;
}

void nesf_default_ai_params(nesf_interface_params* p) {
    nesf_default_ao_params(p);
    default_fluxes(&p->fluxes, true);
    p->humidity_phase = NESF_PHASE_ICE;          // component_interfaces.jl:280-281
    p->has_water_mole_fraction = 0;
    p->water_mole_fraction = 1;
    p->temperature_formulation = NESF_SKIN_TEMPERATURE_CONDUCTIVE;   // sea_ice_simulation.jl:240-249
    p->ice_conductivity = 2;
    p->snow_conductivity = 0.31;
    p->has_radiation = 1;
    p->albedo = 0.7;                             // prescribed_radiation.jl:53-54
    p->emissivity = 1.0;
}

void nesf_default_io_params(nesf_io_params* p) {
    memset(p, 0, sizeof *p);
    p->formulation = 0;                          // ThreeEquationHeatFlux(sea_ice)
    p->conductive = 1;
    p->heat_transfer_coefficient = 0.0095;
    p->salt_transfer_coefficient = 0.0095 / 35;
    p->friction_velocity = 0.002;
    p->ice_conductivity = 2;
    p->reference_latent_heat = 334e3;
    p->liquidus_freshwater_melting_temperature = 0;
    p->liquidus_slope = 0.054;
    p->ocean_reference_density = 1020;
    p->ocean_heat_capacity = 3991.86795711963;
    p->dt = 300;
    p->nz = 1;
    p->stride_k = 0;
}

void nesf_default_assembly_params(nesf_assembly_params* p) {
    p->ocean_reference_density = 1020;
    p->ocean_heat_capacity = 3991.86795711963;
    p->interface_temperature_offset = 273.15;
    p->stefan_boltzmann_constant = 5.670374419e-8;
    p->ocean_albedo = 0.05;
    p->ocean_emissivity = 0.97;
    p->ice_albedo = 0.7;
    p->ice_emissivity = 1.0;
}

void nesf_default_solver_options(nesf_solver_options* o) {
    memset(o, 0, sizeof *o);
    o->precision = NESF_PLAIN_F64;
    o->polish_maxiter = 3;
    o->block_size = 128;
    o->schedule = 0;
    o->ctas_per_sm = 0;
    o->warm_start = 0;
    o->mlp = nullptr;
    o->fallback_ratio = 10.0;
    o->path_tolerance = 2e-6;
    o->fp32_rho = 0.9;
    o->calm_replay_wind = 0.0;
}

// ---------------------------------------------------------------- context
int nesf_context_create(int32_t device, nesf_context** out) {
    if (!out) return fail(NESF_ERR_ARG, "nesf_context_create: null output pointer");
    *out = nullptr;
    int n = 0;
    NESF_CUDA(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return fail(NESF_ERR_ARG, "nesf_context_create: device %d of %d", device, n);
    DeviceGuard g(device);
    if (!g.ok) return fail(NESF_ERR_CUDA, "nesf_context_create: cannot select device %d", device);
    nesf_context* c = new (std::nothrow) nesf_context();
    if (!c) return fail(NESF_ERR_ARG, "nesf_context_create: out of host memory");
    c->device = device;
    c->capacity_members = 0;
    c->d_p64 = nullptr;
    c->d_p32 = nullptr;
    c->d_replay = nullptr;
    c->replay_capacity = 0;
    c->d_pstate = nullptr;
    c->pstate_capacity = 0;
    c->d_work = nullptr;
    c->d_work_count = nullptr;
    c->work_capacity = 0;
    c->work_members = 0;
    c->d_partials = nullptr;
    c->d_feat = nullptr;
    c->d_guess = nullptr;
    c->d_anchor = nullptr;
    c->anchor_capacity = 0;
    c->warm_capacity = 0;
    c->aux = nullptr;
    c->side = nullptr;
    c->ev_fork = c->ev_ice = c->ev_join = c->ev_ocean = nullptr;
    c->tail = nullptr;
    c->ev_tail_fork = c->ev_tail_join = nullptr;
    c->early = nullptr;
    c->ev_early_fork = c->ev_early_join = nullptr;
    c->tuning = default_tuning();
    c->trace = nullptr;
    c->trace_owned = false;
    cudaError_t e = cudaMalloc(&c->d_stats, sizeof(DevStats));
    if (e == cudaSuccess) e = cudaMalloc(&c->d_partials, (size_t)kIntegralBlocks * NESF_MAX_INTEGRALS * 16);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_replay_count, 8 * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMallocHost(&c->h_stats, sizeof(DevStats));
    if (e != cudaSuccess) {
        cudaFree(c->d_stats);
        cudaFree(c->d_partials);
        cudaFree(c->d_replay_count);
        delete c;
        return cuda_fail(e, "nesf_context_create");
    }
    *out = c;
    return NESF_OK;
}

int nesf_context_destroy(nesf_context* c) {
    if (!c) return NESF_OK;
    {
        DeviceGuard g(c->device);
        cudaFree(c->d_stats);
        cudaFreeHost(c->h_stats);
        cudaFree(c->d_p64);
        cudaFree(c->d_p32);
        cudaFree(c->d_replay);
        cudaFree(c->d_pstate);
        cudaFree(c->d_replay_count);
        cudaFree(c->d_work);
        cudaFree(c->d_work_count);
        cudaFree(c->d_partials);
        cudaFree(c->d_feat);
        cudaFree(c->d_guess);
        cudaFree(c->d_anchor);
        if (c->side) cudaStreamDestroy(c->side);
        if (c->ev_fork) cudaEventDestroy(c->ev_fork);
        if (c->ev_ice) cudaEventDestroy(c->ev_ice);
        if (c->ev_ocean) cudaEventDestroy(c->ev_ocean);
        if (c->ev_join) cudaEventDestroy(c->ev_join);
        if (c->tail) cudaStreamDestroy(c->tail);
        if (c->ev_tail_fork) cudaEventDestroy(c->ev_tail_fork);
        if (c->ev_tail_join) cudaEventDestroy(c->ev_tail_join);
        if (c->early) cudaStreamDestroy(c->early);
        if (c->ev_early_fork) cudaEventDestroy(c->ev_early_fork);
        if (c->ev_early_join) cudaEventDestroy(c->ev_early_join);
        if (c->trace && c->trace_owned) {
            for (int i = 0; i < NESF_TRACE_MAX; i++) cudaEventDestroy(c->trace->ev[i]);
            delete c->trace;
        }
    }
    if (c->aux) nesf_context_destroy(c->aux);
    delete c;
    return NESF_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ helpers
static int check_grid(const nesf_grid& g, int hmin, const char* who) {
    if (g.nx <= 0 || g.ny <= 0) return fail(NESF_ERR_ARG, "%s: grid size %d x %d", who, g.nx, g.ny);
    if (g.hx < hmin || g.hy < hmin)
        return fail(NESF_ERR_ARG, "%s: halo (%d, %d) smaller than %d", who, g.hx, g.hy, hmin);
    if (g.stride_j < (int64_t)g.nx + 2 * g.hx)
        return fail(NESF_ERR_ARG, "%s: stride_j %lld < nx + 2hx", who, (long long)g.stride_j);
    return NESF_OK;
}

static Layout2 layout(const nesf_grid& g) { return Layout2{g.nx, g.ny, g.hx, g.hy, g.stride_j}; }

static int check_params(const nesf_interface_params* p, const char* who) {
    if (!p) return fail(NESF_ERR_ARG, "%s: null params", who);
    const nesf_similarity_theory_fluxes& f = p->fluxes;
    if (f.maxiter < 0) return fail(NESF_ERR_ARG, "%s: maxiter %d < 0", who, f.maxiter);
    if (!(f.tolerance >= 0)) return fail(NESF_ERR_ARG, "%s: tolerance must be >= 0", who);
    for (int n = 0; n < 3; n++) {
        if (f.stability[n].kind < NESF_PSI_ZERO || f.stability[n].kind > NESF_PSI_LINEAR_PAULSON_SCALAR)
            return fail(NESF_ERR_ARG, "%s: stability function kind %d", who, f.stability[n].kind);
        if (f.roughness[n].kind < NESF_ROUGHNESS_CONSTANT || f.roughness[n].kind > NESF_ROUGHNESS_SCALAR)
            return fail(NESF_ERR_ARG, "%s: roughness kind %d", who, f.roughness[n].kind);
    }
    if (f.roughness[0].kind == NESF_ROUGHNESS_SCALAR)
        return fail(NESF_ERR_ARG, "%s: the momentum roughness cannot be a ScalarRoughnessLength", who);
    if (p->temperature_formulation < NESF_BULK_TEMPERATURE ||
        p->temperature_formulation > NESF_SKIN_TEMPERATURE_DIFFUSIVE)
        return fail(NESF_ERR_ARG, "%s: temperature formulation %d", who, p->temperature_formulation);
    if (p->surface_layer_height <= 0) return fail(NESF_ERR_ARG, "%s: surface_layer_height <= 0", who);
    if (p->humidity_formulation < NESF_HUMIDITY_IMPURE_SATURATION || p->humidity_formulation > NESF_HUMIDITY_DRY_LAYER)
        return fail(NESF_ERR_ARG, "%s: humidity formulation %d", who, p->humidity_formulation);
    if (p->flux_formulation != NESF_FLUXES_SIMILARITY_THEORY && p->flux_formulation != NESF_FLUXES_COEFFICIENT_BASED)
        return fail(NESF_ERR_ARG, "%s: flux formulation %d", who, p->flux_formulation);
    if (p->flux_formulation == NESF_FLUXES_COEFFICIENT_BASED) {
        const nesf_coefficient_fluxes& c = p->coefficients;
        if (c.kind != NESF_COEFFICIENTS_CONSTANT && c.kind != NESF_COEFFICIENTS_LARGE_YEAGER)
            return fail(NESF_ERR_ARG, "%s: transfer coefficients kind %d", who, c.kind);
        if (c.maxiter < 0 || !(c.tolerance >= 0))
            return fail(NESF_ERR_ARG, "%s: coefficient-based stop criteria (maxiter %d, tolerance %g)", who,
                        c.maxiter, c.tolerance);
        if (c.kind == NESF_COEFFICIENTS_LARGE_YEAGER) {
            if (!(c.reference_height > 0) || !(c.von_karman_constant > 0))
                return fail(NESF_ERR_ARG, "%s: Large-Yeager reference height and von Karman constant must be > 0",
                            who);
            for (int n = 0; n < 2; n++)
                if (c.stability[n].kind < NESF_PSI_ZERO || c.stability[n].kind > NESF_PSI_LINEAR_PAULSON_SCALAR)
                    return fail(NESF_ERR_ARG, "%s: stability function kind %d", who, c.stability[n].kind);
        }
    }
    return NESF_OK;
}

static nesf_solver_options options_or_default(const nesf_solver_options* o) {
    nesf_solver_options d;
    nesf_default_solver_options(&d);
    if (!o) return d;
    nesf_solver_options r = *o;
    if (r.polish_maxiter <= 0) r.polish_maxiter = d.polish_maxiter;
    if (!(r.path_tolerance > 0)) r.path_tolerance = d.path_tolerance;
    if (!(r.fp32_rho > 0)) r.fp32_rho = d.fp32_rho;
    if (!(r.fallback_ratio > 0)) r.fallback_ratio = d.fallback_ratio;
    return r;
}

// The kernels' knobs; fp32_rho = 0 keeps no FP32 result (NESF_F32_POLISH). Launch
// shapes from the context's tuning (the defaults without a context).
static SolveOpts solve_opts(const nesf_solver_options& o, const nesf_context* ctx = nullptr) {
    float rho = o.precision == NESF_F32_ADAPTIVE ? (float)(o.fp32_rho < 0.99 ? o.fp32_rho : 0.99) : 0.0f;
    const nesf_tuning t = ctx ? ctx->tuning : default_tuning();
    return SolveOpts{o.polish_maxiter, (float)o.path_tolerance, rho, (float)o.fallback_ratio,
                     t.solve_block, t.deferred_per_sm, t.infer_per_sm,
                     (t.pass1_fetch >= 2 ? NESF_FETCH_SEA_ICE : 0) | (t.pass1_fetch >= 3 ? NESF_FETCH_OCEAN : 0),
                     t.pass1_fetch == 4 ? (t.refill_lanes > 0 ? t.refill_lanes : 8) : 32, tracer_of(ctx),
                     (float)o.calm_replay_wind, t.ice_deferred_per_sm > 0 ? t.ice_deferred_per_sm : t.deferred_per_sm,
                     t.cells_per_thread > 0 ? t.cells_per_thread : 1};
}

static int check_options(const nesf_solver_options& o, const char* who) {
    if (o.precision != NESF_PLAIN_F64 && o.precision != NESF_F32_POLISH && o.precision != NESF_F32_ADAPTIVE)
        return fail(NESF_ERR_ARG, "%s: precision %d", who, o.precision);
    if (o.warm_start && !o.mlp) return fail(NESF_ERR_ARG, "%s: warm_start without a network (mlp)", who);
    if (o.warm_start && !(o.fallback_ratio > 0)) return fail(NESF_ERR_ARG, "%s: fallback_ratio must be > 0", who);
    if (!(o.calm_replay_wind >= 0) || o.calm_replay_wind > 1e3)
        return fail(NESF_ERR_ARG, "%s: calm_replay_wind %g (0..1000 m/s)", who, o.calm_replay_wind);
    return NESF_OK;
}

// The context's queues of deferred cells (replay and polish), grown to `cells`
// entries each (caller holds ctx->lock). Growing synchronises the device: size
// the first call for the largest grid.
static int replay_queue(nesf_context* ctx, int64_t cells, ReplayQueue* q, bool with_state = false) {
    if (cells > ctx->replay_capacity) {
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) return cuda_fail(e, "replay queue");
        cudaFree(ctx->d_replay);
        ctx->d_replay = nullptr;
        ctx->replay_capacity = 0;
        NESF_CUDA(cudaMalloc(&ctx->d_replay, 4 * sizeof(uint32_t) * (size_t)cells));
        ctx->replay_capacity = cells;
    }
    // the polish state (sea-ice solves): one entry per polish-queue entry, so that every
    // polished cell takes the same path whatever its position in the queue
    if (with_state && ctx->pstate_capacity < ctx->replay_capacity) {
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) return cuda_fail(e, "polish state");
        cudaFree(ctx->d_pstate);
        ctx->d_pstate = nullptr;
        ctx->pstate_capacity = 0;
        NESF_CUDA(cudaMalloc(&ctx->d_pstate, sizeof(float) * kPolishStateFloats * (size_t)ctx->replay_capacity));
        ctx->pstate_capacity = ctx->replay_capacity;
    }
    q->idx = ctx->d_replay;
    q->count = ctx->d_replay_count;
    q->capacity = ctx->replay_capacity;
    q->pstate = with_state ? ctx->d_pstate : nullptr;
    return NESF_OK;
}

// The sea-ice solve's second and third streams for its deferred passes and its calm
// cells' early replays (created once; before a graph capture by coupling_scratch).
static int tail_lane(nesf_context* ctx) {
    if (ctx->tail && ctx->early) return NESF_OK;
    DeviceGuard g(ctx->device);
    if (!ctx->tail) {
        NESF_CUDA(cudaEventCreateWithFlags(&ctx->ev_tail_fork, cudaEventDisableTiming));
        NESF_CUDA(cudaEventCreateWithFlags(&ctx->ev_tail_join, cudaEventDisableTiming));
        NESF_CUDA(cudaStreamCreateWithFlags(&ctx->tail, cudaStreamNonBlocking));
    }
    NESF_CUDA(cudaEventCreateWithFlags(&ctx->ev_early_fork, cudaEventDisableTiming));
    NESF_CUDA(cudaEventCreateWithFlags(&ctx->ev_early_join, cudaEventDisableTiming));
    NESF_CUDA(cudaStreamCreateWithFlags(&ctx->early, cudaStreamNonBlocking));
    return NESF_OK;
}

// The context's work lists: `members` segments of `per_member` entries.
static int work_list(nesf_context* ctx, int64_t per_member, int32_t members, WorkList* w) {
    int64_t need = per_member * members;
    if (need > ctx->work_capacity || members > ctx->work_members) {
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) return cuda_fail(e, "work list");
        cudaFree(ctx->d_work);
        cudaFree(ctx->d_work_count);
        ctx->d_work = nullptr;
        ctx->d_work_count = nullptr;
        ctx->work_capacity = 0;
        ctx->work_members = 0;
        int64_t cap = need > ctx->work_capacity ? need : ctx->work_capacity;
        int32_t mem = members > ctx->work_members ? members : ctx->work_members;
        NESF_CUDA(cudaMalloc(&ctx->d_work, sizeof(uint32_t) * (size_t)cap));
        NESF_CUDA(cudaMalloc(&ctx->d_work_count, sizeof(unsigned int) * 2 * (size_t)mem));
        ctx->work_capacity = cap;
        ctx->work_members = mem;
    }
    w->idx = ctx->d_work;
    w->count = ctx->d_work_count;
    w->per_member = per_member;
    return NESF_OK;
}

// Library-owned context of the current device, for calls that pass none.
static nesf_context* g_default_ctx[64];
static std::mutex g_default_lock;

// The context's warm-start buffers for `cells` work-list slots (caller holds the lock).
static int warm_buffers(nesf_context* ctx, const nesf_solver_options& o, int64_t cells, WarmStart* ws) {
    *ws = WarmStart{nullptr, nullptr, nullptr, nullptr};
    // the adaptive solver's per-slot records of the cancelling differences (classify -> pass 1)
    if (o.precision == NESF_F32_ADAPTIVE) {
        if (cells > ctx->anchor_capacity) {
            cudaError_t e = cudaDeviceSynchronize();
            if (e != cudaSuccess) return cuda_fail(e, "anchor buffer");
            cudaFree(ctx->d_anchor);
            ctx->d_anchor = nullptr;
            ctx->anchor_capacity = 0;
            NESF_CUDA(cudaMalloc(&ctx->d_anchor, sizeof(float) * kAnchorFloats * (size_t)cells));
            ctx->anchor_capacity = cells;
        }
        ws->anc = ctx->d_anchor;
    }
    if (!o.warm_start || o.precision == NESF_PLAIN_F64) return NESF_OK;
    if (cells > ctx->warm_capacity) {
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) return cuda_fail(e, "warm-start buffers");
        cudaFree(ctx->d_feat);
        cudaFree(ctx->d_guess);
        ctx->d_feat = ctx->d_guess = nullptr;
        ctx->warm_capacity = 0;
        NESF_CUDA(cudaMalloc(&ctx->d_feat, sizeof(float) * 8 * (size_t)cells));
        NESF_CUDA(cudaMalloc(&ctx->d_guess, sizeof(float) * 4 * (size_t)cells));
        ctx->warm_capacity = cells;
    }
    ws->feat = ctx->d_feat;
    ws->guess = ctx->d_guess;
    ws->mlp = o.mlp;
    return NESF_OK;
}

static int context_or_default(nesf_context** ctx) {
    if (*ctx) return NESF_OK;
    int dev = 0;
    NESF_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(NESF_ERR_ARG, "device %d", dev);
    std::lock_guard<std::mutex> lk(g_default_lock);
    if (!g_default_ctx[dev]) {
        int r = nesf_context_create(dev, &g_default_ctx[dev]);
        if (r) return r;
    }
    *ctx = g_default_ctx[dev];
    return NESF_OK;
}

// cpu_interpolating_time_indices of a FieldTimeSeries (interpolate_atmospheric_state.jl:57-60):
// the bracketing snapshots of t and the weight of the second, on the host.
int nesf_time_indices(const double* times, int32_t nt, int32_t indexing, double period, double t, int32_t* n1,
                      int32_t* n2, double* weight) {
    const char* who = "nesf_time_indices";
    if (!times || !n1 || !n2 || !weight || nt < 1) return fail(NESF_ERR_ARG, "%s: null argument or nt < 1", who);
    if (indexing < NESF_TIME_CYCLICAL || indexing > NESF_TIME_CLAMP)
        return fail(NESF_ERR_ARG, "%s: time indexing %d", who, indexing);
    if (!std::isfinite(t)) return fail(NESF_ERR_ARG, "%s: time %g", who, t);
    for (int32_t n = 1; n < nt; n++)
        if (!(times[n] > times[n - 1])) return fail(NESF_ERR_ARG, "%s: times not strictly increasing at %d", who, n);
    if (nt == 1) {
        *n1 = *n2 = 0;
        *weight = 0;
        return NESF_OK;
    }
    const double t0 = times[0], tl = times[nt - 1];
    if (indexing == NESF_TIME_CYCLICAL) {
        const double P = period > 0 ? period : (tl - t0) + (tl - times[nt - 2]);
        if (!(P > tl - t0)) return fail(NESF_ERR_ARG, "%s: period %g does not exceed the times' span", who, P);
        double tau = std::fmod(t - t0, P);
        if (tau < 0) tau += P;
        t = t0 + tau;
        if (t >= tl) {   // between the last snapshot and the first one's next cycle
            *n1 = nt - 1;
            *n2 = 0;
            *weight = (t - tl) / (t0 + P - tl);
            return NESF_OK;
        }
    } else if (indexing == NESF_TIME_CLAMP && (t <= t0 || t >= tl)) {
        *n1 = *n2 = t <= t0 ? 0 : nt - 1;
        *weight = 0;
        return NESF_OK;
    }
    // the last snapshot at or before t, within [0, nt - 2]
    int32_t lo = 0, hi = nt - 1;
    if (t < t0) hi = 0;
    while (hi - lo > 1) {
        const int32_t mid = lo + (hi - lo) / 2;
        if (times[mid] <= t) lo = mid;
        else hi = mid;
    }
    const int32_t n = lo < nt - 2 ? lo : nt - 2;
    *n1 = n;
    *n2 = n + 1;
    *weight = (t - times[n]) / (times[n + 1] - times[n]);
    return NESF_OK;
}

// The library's per-device set-up done ahead of the first call: the default context of
// `device` (its streams, events and scratch), which the calls that take a null context
// use. The caller's current device is left as it was.
int nesf_init(int32_t device) {
    int n = 0;
    NESF_CUDA(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n || device >= 64) return fail(NESF_ERR_ARG, "nesf_init: device %d of %d", device, n);
    std::lock_guard<std::mutex> lk(g_default_lock);
    if (!g_default_ctx[device]) return nesf_context_create(device, &g_default_ctx[device]);
    return NESF_OK;
}

static void stats_to_public(const DevStats& d, nesf_stats* s) {
    s->cells = (int64_t)d.cells;
    s->solved = (int64_t)d.solved;
    s->iterations = (int64_t)d.iterations;
    s->max_iterations = (int64_t)d.max_iterations;
    s->nonconverged = (int64_t)d.nonconverged;
    s->polished = (int64_t)d.polished;
    s->polish_iterations = (int64_t)d.polish_iterations;
    s->cold_fallbacks = (int64_t)d.cold_fallbacks;
    s->fp64_redo = (int64_t)d.fp64_redo;
    for (int k = 0; k < 5; k++) s->replay_reasons[k] = (int64_t)d.replay_reasons[k];
    for (int k = 0; k < NESF_ITER_HIST_BINS; k++) s->histogram[k] = (int64_t)d.hist[k];
}

// Runs `launch(d_stats or nullptr)` with optional statistics readback.
template <class F>
static int with_stats(nesf_context* ctx, nesf_stats* stats, cudaStream_t s, F launch) {
    DevStats* ds = nullptr;
    if (stats) {
        ds = ctx->d_stats;
        NESF_CUDA(cudaMemsetAsync(ds, 0, sizeof(DevStats), s));
    }
    cudaError_t e = launch(ds);
    if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
    if (stats) {
        NESF_CUDA(cudaMemcpyAsync(ctx->h_stats, ds, sizeof(DevStats), cudaMemcpyDeviceToHost, s));
        NESF_CUDA(cudaStreamSynchronize(s));
        stats_to_public(*ctx->h_stats, stats);
    }
    return NESF_OK;
}

template <class S>
static AOArgs<S> ao_args(const nesf_ao_fields* f, int64_t member_stride) {
    AOArgs<S> a;
    a.L = layout(f->grid);
    a.member_stride = member_stride;
    a.ua = (const S*)f->u_atm; a.va = (const S*)f->v_atm; a.Ta = (const S*)f->T_atm;
    a.pa = (const S*)f->p_atm; a.qa = (const S*)f->q_atm;
    a.uo = (const S*)f->u_oc; a.vo = (const S*)f->v_oc; a.To = (const S*)f->T_oc; a.So = (const S*)f->S_oc;
    a.inactive = f->inactive;
    a.sw = (const S*)f->sw_down; a.lw = (const S*)f->lw_down; a.kappa = (const S*)f->kappa;
    a.Qv = (S*)f->latent_heat; a.QT = (S*)f->sensible_heat; a.Jv = (S*)f->water_vapor;
    a.tx = (S*)f->x_momentum; a.ty = (S*)f->y_momentum;
    a.us = (S*)f->friction_velocity; a.ts = (S*)f->temperature_scale; a.qs = (S*)f->water_vapor_scale;
    a.Ts = (S*)f->interface_temperature;
    a.iters = f->iterations;
    return a;
}

static int check_ao_fields(const nesf_ao_fields* f, const nesf_interface_params* p, const char* who) {
    if (!f) return fail(NESF_ERR_ARG, "%s: null fields", who);
    if (p->humidity_formulation != NESF_HUMIDITY_IMPURE_SATURATION)
        return fail(NESF_ERR_UNSUPPORTED, "%s: the ocean surface humidity is ImpureSaturationSpecificHumidity", who);
    int r = check_grid(f->grid, 2, who);
    if (r) return r;
    if (f->dtype != NESF_F64 && f->dtype != NESF_F32) return fail(NESF_ERR_ARG, "%s: dtype %d", who, f->dtype);
    const void* req[] = {f->u_atm, f->v_atm, f->T_atm, f->p_atm, f->q_atm, f->u_oc, f->v_oc, f->T_oc, f->S_oc};
    const char* names[] = {"u_atm", "v_atm", "T_atm", "p_atm", "q_atm", "u_oc", "v_oc", "T_oc", "S_oc"};
    for (int k = 0; k < 9; k++)
        if (!req[k]) return fail(NESF_ERR_ARG, "%s: required input %s is NULL", who, names[k]);
    if (p->temperature_formulation == NESF_SKIN_TEMPERATURE_CONDUCTIVE)
        return fail(NESF_ERR_UNSUPPORTED, "%s: conductive skin temperature over the ocean", who);
    if (p->has_radiation && p->temperature_formulation != NESF_BULK_TEMPERATURE && (!f->sw_down || !f->lw_down))
        return fail(NESF_ERR_ARG, "%s: skin temperature with radiation needs sw_down and lw_down", who);
    return NESF_OK;
}

// The atmosphere-ocean solve; before_pass1 (optional): an event its stream waits for after the
// classify pass and the warm-start inference, before pass 1; mid (optional): recorded on the
// stream after the inference, then its hook enqueues work of another lane (which may wait for
// the event), before the wait for before_pass1 is enqueued.
static int ocean_fluxes(nesf_context* ctx, const nesf_interface_params* params, const nesf_ao_fields* f,
                        const nesf_solver_options* opts, nesf_stats* stats, void* stream, cudaEvent_t before_pass1,
                        MidHook* mid = nullptr) {
    const char* who = "nesf_compute_atmosphere_ocean_fluxes";
    int r = check_params(params, who);
    if (r) return r;
    if ((r = check_ao_fields(f, params, who))) return r;
    nesf_solver_options o = options_or_default(opts);
    if ((r = check_options(o, who))) return r;
    if ((r = context_or_default(&ctx))) return r;
    std::lock_guard<std::mutex> lk(ctx->lock);
    DeviceGuard g(ctx->device);
    DevIface<double> P64 = make_dev_iface<double>(*params);
    DevIface<float> P32 = make_dev_iface<float>(*params);
    cudaStream_t s = (cudaStream_t)stream;
    bool skin = params->temperature_formulation != NESF_BULK_TEMPERATURE;
    int64_t ring = (int64_t)(f->grid.nx + 2) * (f->grid.ny + 2);
    ReplayQueue rq;
    WorkList wl;
    WarmStart ws;
    if ((r = replay_queue(ctx, ring, &rq))) return r;
    if ((r = work_list(ctx, ring, 1, &wl))) return r;
    if ((r = warm_buffers(ctx, o, ring, &ws))) return r;
    SolveOpts so = solve_opts(o, ctx);
    const DevIface<df> Pdf = make_dev_iface<df>(*params);
    so.pdf = &Pdf;
    // pass 1's replays beside the polish pass (the tuning's two_lanes)
    TailLane tl{nullptr, nullptr, nullptr};
    if (o.precision == NESF_F32_ADAPTIVE && ctx->tuning.two_lanes) {
        if ((r = tail_lane(ctx))) return r;
        tl = TailLane{ctx->tail, ctx->ev_tail_fork, ctx->ev_tail_join};
    }
    return with_stats(ctx, stats, s, [&](DevStats* ds) {
        if (f->dtype == NESF_F64)
            return launch_ao(ao_args<double>(f, 0), P64, P32, nullptr, nullptr, 1, o.precision, skin, so, wl, rq, ws,
                             ds, s, before_pass1, &tl, mid);
        return launch_ao(ao_args<float>(f, 0), P64, P32, nullptr, nullptr, 1, o.precision, skin, so, wl, rq, ws, ds,
                         s, before_pass1, &tl, mid);
    });
}

extern "C" int nesf_compute_atmosphere_ocean_fluxes(nesf_context* ctx, const nesf_interface_params* params,
                                                    const nesf_ao_fields* f, const nesf_solver_options* opts,
                                                    nesf_stats* stats, void* stream) {
    return ocean_fluxes(ctx, params, f, opts, stats, stream, nullptr);
}

extern "C" int nesf_compute_atmosphere_ocean_fluxes_ensemble(nesf_context* ctx, const nesf_interface_params* params,
                                                             int32_t members, int64_t member_stride,
                                                             const nesf_ao_fields* f,
                                                             const nesf_solver_options* opts, nesf_stats* stats,
                                                             void* stream) {
    const char* who = "nesf_compute_atmosphere_ocean_fluxes_ensemble";
    if (!ctx) return fail(NESF_ERR_ARG, "%s: needs a context", who);
    if (members <= 0 || members > 65535) return fail(NESF_ERR_ARG, "%s: members = %d", who, members);
    int r;
    for (int m = 0; m < members; m++)
        if ((r = check_params(params + m, who))) return r;
    if ((r = check_ao_fields(f, params, who))) return r;
    for (int m = 1; m < members; m++)
        if (params[m].temperature_formulation != params[0].temperature_formulation)
            return fail(NESF_ERR_ARG, "%s: members must share the temperature formulation", who);
    int64_t plane = f->grid.stride_j * ((int64_t)f->grid.ny + 2 * f->grid.hy);
    if (member_stride < plane) return fail(NESF_ERR_ARG, "%s: member_stride smaller than one array", who);
    nesf_solver_options o = options_or_default(opts);
    if ((r = check_options(o, who))) return r;
    std::lock_guard<std::mutex> lk(ctx->lock);
    DeviceGuard g(ctx->device);
    cudaStream_t s = (cudaStream_t)stream;
    if (members > ctx->capacity_members) {
        cudaFree(ctx->d_p64);
        cudaFree(ctx->d_p32);
        ctx->d_p64 = nullptr;
        ctx->d_p32 = nullptr;
        ctx->capacity_members = 0;
        NESF_CUDA(cudaMalloc(&ctx->d_p64, sizeof(DevIface<double>) * members));
        NESF_CUDA(cudaMalloc(&ctx->d_p32, sizeof(DevIface<float>) * members));
        ctx->capacity_members = members;
    }
    DevIface<double>* h64 = new DevIface<double>[members];
    DevIface<float>* h32 = new DevIface<float>[members];
    for (int m = 0; m < members; m++) {
        h64[m] = make_dev_iface<double>(params[m]);
        h32[m] = make_dev_iface<float>(params[m]);
    }
    cudaError_t e = cudaMemcpyAsync(ctx->d_p64, h64, sizeof(DevIface<double>) * members, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx->d_p32, h32, sizeof(DevIface<float>) * members, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);   // host staging buffers are freed below
    delete[] h64;
    delete[] h32;
    if (e != cudaSuccess) return cuda_fail(e, who);
    DevIface<double> P64 = make_dev_iface<double>(params[0]);
    DevIface<float> P32 = make_dev_iface<float>(params[0]);
    bool skin = params->temperature_formulation != NESF_BULK_TEMPERATURE;
    int64_t ring = (int64_t)(f->grid.nx + 2) * (f->grid.ny + 2);
    if (ring * members > 0xffffffffLL) return fail(NESF_ERR_CAPACITY, "%s: too many cells for the queue", who);
    ReplayQueue rq;
    WorkList wl;
    if ((r = replay_queue(ctx, ring * members, &rq))) return r;
    if ((r = work_list(ctx, ring, members, &wl))) return r;
    SolveOpts so = solve_opts(o, ctx);
    return with_stats(ctx, stats, s, [&](DevStats* ds) {
        if (f->dtype == NESF_F64)
            return launch_ao(ao_args<double>(f, member_stride), P64, P32, ctx->d_p64, ctx->d_p32, members,
                             o.precision, skin, so, wl, rq, WarmStart{}, ds, s);
        return launch_ao(ao_args<float>(f, member_stride), P64, P32, ctx->d_p64, ctx->d_p32, members, o.precision,
                         skin, so, wl, rq, WarmStart{}, ds, s);
    });
}

template <class S>
static AIArgs<S> ai_args(const nesf_ai_fields* f) {
    AIArgs<S> a;
    a.L = layout(f->grid);
    a.ua = (const S*)f->u_atm; a.va = (const S*)f->v_atm; a.Ta = (const S*)f->T_atm;
    a.pa = (const S*)f->p_atm; a.qa = (const S*)f->q_atm;
    a.To = (const S*)f->T_oc; a.So = (const S*)f->S_oc;
    a.hi = (const S*)f->ice_thickness; a.hs = (const S*)f->snow_thickness;
    a.hc = (const S*)f->consolidation_thickness; a.aleph = (const S*)f->ice_concentration;
    a.inactive = f->inactive;
    a.sw = (const S*)f->sw_down; a.lw = (const S*)f->lw_down;
    a.Ts = (S*)f->interface_temperature;
    a.Qv = (S*)f->latent_heat; a.QT = (S*)f->sensible_heat; a.Jv = (S*)f->water_vapor;
    a.tx = (S*)f->x_momentum; a.ty = (S*)f->y_momentum;
    a.iters = f->iterations;
    return a;
}

template <class S>
static ALArgs<S> al_args(const nesf_al_fields* f) {
    ALArgs<S> a;
    a.L = layout(f->grid);
    a.ua = (const S*)f->u_atm; a.va = (const S*)f->v_atm; a.Ta = (const S*)f->T_atm;
    a.pa = (const S*)f->p_atm; a.qa = (const S*)f->q_atm;
    a.T = (const S*)f->land_temperature; a.sat = (const S*)f->saturation;
    a.Qv = (S*)f->latent_heat; a.QT = (S*)f->sensible_heat; a.Jv = (S*)f->water_vapor;
    a.tx = (S*)f->x_momentum; a.ty = (S*)f->y_momentum;
    a.us = (S*)f->friction_velocity; a.ts = (S*)f->temperature_scale; a.qs = (S*)f->water_vapor_scale;
    a.Ts = (S*)f->interface_temperature;
    a.iters = f->iterations;
    return a;
}

extern "C" int nesf_compute_atmosphere_land_fluxes(nesf_context* ctx, const nesf_interface_params* params,
                                                   const nesf_al_fields* f, const nesf_solver_options* opts,
                                                   nesf_stats* stats, void* stream) {
    const char* who = "nesf_compute_atmosphere_land_fluxes";
    int r = check_params(params, who);
    if (r) return r;
    if (!f) return fail(NESF_ERR_ARG, "%s: null fields", who);
    if ((r = check_grid(f->grid, 0, who))) return r;
    if (f->dtype != NESF_F64 && f->dtype != NESF_F32) return fail(NESF_ERR_ARG, "%s: dtype %d", who, f->dtype);
    const void* req[] = {f->u_atm, f->v_atm, f->T_atm, f->p_atm, f->q_atm, f->land_temperature};
    for (const void* q : req)
        if (!q) return fail(NESF_ERR_ARG, "%s: a required array is NULL", who);
    if (params->temperature_formulation != NESF_BULK_TEMPERATURE)
        return fail(NESF_ERR_UNSUPPORTED, "%s: the land interface takes BulkTemperature", who);
    const int hf = params->humidity_formulation;
    if ((hf == NESF_HUMIDITY_BULK || hf == NESF_HUMIDITY_DRY_LAYER ||
         (hf == NESF_HUMIDITY_FRACTIONAL && params->critical_saturation > 0)) &&
        !f->saturation)
        return fail(NESF_ERR_ARG, "%s: the humidity model needs the land saturation", who);
    if (hf == NESF_HUMIDITY_SKIN && !(params->skin_surface_thickness > 0 && params->skin_vapor_diffusivity >= 0))
        return fail(NESF_ERR_ARG, "%s: SkinHumidity needs surface_thickness > 0 and vapor_diffusivity >= 0", who);
    // DryLayerHumidity: the reference accepts any numbers; a zero minimum depth, onset saturation
    // or exchange depth divides by zero (0/0 where the layer is wet) and a zero porosity does
    // under the power-law tortuosity, so these are rejected rather than turned into NaN fields.
    if (hf == NESF_HUMIDITY_DRY_LAYER) {
        const nesf_interface_params& q = *params;
        if (q.tortuosity != NESF_TORTUOSITY_CONSTANT && q.tortuosity != NESF_TORTUOSITY_POWER_LAW)
            return fail(NESF_ERR_ARG, "%s: tortuosity %d", who, q.tortuosity);
        if (!(q.maximum_dry_layer_depth >= 0 && q.dry_layer_onset_saturation > 0 && q.minimum_dry_layer_depth > 0 &&
              q.molecular_diffusivity >= 0 && q.wet_transition_width >= 0 && q.thermal_exchange_depth > 0 &&
              std::isfinite(q.dry_layer_exponent) &&
              (q.tortuosity == NESF_TORTUOSITY_CONSTANT || q.porosity > 0)))
            return fail(NESF_ERR_ARG,
                        "%s: DryLayerHumidity needs maximum depth >= 0, onset saturation > 0, minimum depth > 0, "
                        "diffusivity >= 0, transition width >= 0, exchange depth > 0 and (power law) porosity > 0",
                        who);
    }
    nesf_solver_options o = options_or_default(opts);
    if ((r = check_options(o, who))) return r;
    if ((r = context_or_default(&ctx))) return r;
    std::lock_guard<std::mutex> lk(ctx->lock);
    DeviceGuard g(ctx->device);
    DevIface<double> P64 = make_dev_iface<double>(*params);
    DevIface<float> P32 = make_dev_iface<float>(*params);
    cudaStream_t s = (cudaStream_t)stream;
    SolveOpts so = solve_opts(o, ctx);
    return with_stats(ctx, stats, s, [&](DevStats* ds) {
        if (f->dtype == NESF_F64) return launch_al(al_args<double>(f), P64, P32, o.precision, so, ds, s);
        return launch_al(al_args<float>(f), P64, P32, o.precision, so, ds, s);
    });
}

// The sea-ice solve; `after_solve` (optional) is recorded on the stream once the
// pass-1 solve is enqueued, before the packed polish and replay passes; `before_pass1`
// (optional) is waited for before pass 1; `mid` (optional): run after pass 1 (MidHook).
static int sea_ice_fluxes(nesf_context* ctx, const nesf_interface_params* params, const nesf_ai_fields* f,
                          const nesf_solver_options* opts, nesf_stats* stats, void* stream,
                          cudaEvent_t after_solve, cudaEvent_t before_pass1 = nullptr, MidHook* mid = nullptr) {
    const char* who = "nesf_compute_atmosphere_sea_ice_fluxes";
    int r = check_params(params, who);
    if (r) return r;
    if (!f) return fail(NESF_ERR_ARG, "%s: null fields", who);
    if ((r = check_grid(f->grid, 1, who))) return r;
    if (f->dtype != NESF_F64 && f->dtype != NESF_F32) return fail(NESF_ERR_ARG, "%s: dtype %d", who, f->dtype);
    const void* req[] = {f->u_atm, f->v_atm, f->T_atm, f->p_atm, f->q_atm, f->T_oc, f->S_oc, f->ice_thickness,
                         f->consolidation_thickness, f->ice_concentration, f->interface_temperature};
    for (const void* q : req)
        if (!q) return fail(NESF_ERR_ARG, "%s: a required array is NULL", who);
    if (params->temperature_formulation == NESF_SKIN_TEMPERATURE_DIFFUSIVE)
        return fail(NESF_ERR_UNSUPPORTED, "%s: diffusive skin temperature over sea ice", who);
    if (params->humidity_formulation != NESF_HUMIDITY_IMPURE_SATURATION)
        return fail(NESF_ERR_UNSUPPORTED, "%s: the sea-ice surface humidity is ImpureSaturationSpecificHumidity", who);
    if (params->temperature_formulation == NESF_SKIN_TEMPERATURE_CONDUCTIVE && params->snow_conductivity > 0 &&
        !f->snow_thickness)
        return fail(NESF_ERR_ARG, "%s: snow conductivity given but snow_thickness is NULL", who);
    if (params->has_radiation && (!f->sw_down || !f->lw_down))
        return fail(NESF_ERR_ARG, "%s: radiation enabled but sw_down/lw_down NULL", who);
    nesf_solver_options o = options_or_default(opts);
    if ((r = check_options(o, who))) return r;
    if ((r = context_or_default(&ctx))) return r;
    std::lock_guard<std::mutex> lk(ctx->lock);
    DeviceGuard g(ctx->device);
    DevIface<double> P64 = make_dev_iface<double>(*params);
    DevIface<float> P32 = make_dev_iface<float>(*params);
    cudaStream_t s = (cudaStream_t)stream;
    int64_t ring = (int64_t)(f->grid.nx + 2) * (f->grid.ny + 2);
    ReplayQueue rq;
    WorkList wl;
    WarmStart ws;
    if ((r = replay_queue(ctx, ring, &rq, true))) return r;
    if ((r = work_list(ctx, ring, 1, &wl))) return r;
    if ((r = warm_buffers(ctx, o, ring, &ws))) return r;
    SolveOpts so = solve_opts(o, ctx);
    const DevIface<df> Pdf = make_dev_iface<df>(*params);
    so.pdf = &Pdf;
    // the replay of pass 1's cells beside the polish pass and the calm cells' replays beside
    // pass 1 (the tuning's two_lanes)
    TailLane tl{nullptr, nullptr, nullptr}, el{nullptr, nullptr, nullptr};
    if (o.precision == NESF_F32_ADAPTIVE && ctx->tuning.two_lanes) {
        if ((r = tail_lane(ctx))) return r;
        tl = TailLane{ctx->tail, ctx->ev_tail_fork, ctx->ev_tail_join};
        el = TailLane{ctx->early, ctx->ev_early_fork, ctx->ev_early_join};
    }
    return with_stats(ctx, stats, s, [&](DevStats* ds) {
        if (f->dtype == NESF_F64)
            return launch_ai(ai_args<double>(f), P64, P32, o.precision, so, wl, rq, ws, ds, s, after_solve, &tl,
                             &el, before_pass1, mid);
        return launch_ai(ai_args<float>(f), P64, P32, o.precision, so, wl, rq, ws, ds, s, after_solve, &tl, &el,
                         before_pass1, mid);
    });
}

extern "C" int nesf_compute_atmosphere_sea_ice_fluxes(nesf_context* ctx, const nesf_interface_params* params,
                                                      const nesf_ai_fields* f, const nesf_solver_options* opts,
                                                      nesf_stats* stats, void* stream) {
    return sea_ice_fluxes(ctx, params, f, opts, stats, stream, nullptr);
}

template <class S>
static IOArgs<S> io_args(const nesf_io_fields* f) {
    IOArgs<S> a;
    a.L = layout(f->grid);
    a.T3 = (S*)f->T_oc; a.S3 = (const S*)f->S_oc; a.dz = f->dz;
    a.Si = (const S*)f->ice_salinity; a.hi = (const S*)f->ice_thickness; a.hc = (const S*)f->consolidation_thickness;
    a.aleph = (const S*)f->ice_concentration; a.Tint = (const S*)f->internal_temperature;
    a.Ei = (const S*)f->ice_mass_flux; a.Es = (const S*)f->snow_mass_flux;
    a.Qio = (S*)f->interface_heat; a.frazil = (S*)f->frazil_heat; a.Js = (S*)f->salt; a.Jw = (S*)f->freshwater;
    a.Tb = (S*)f->interface_T; a.Sb = (S*)f->interface_S;
    return a;
}

// part: 0 fluxes + frazil adjustment of the ocean temperature, 1 the fluxes alone
// (the ocean state read only), 2 the adjustment alone (launch_io).
static int sea_ice_ocean(nesf_context* ctx, const nesf_io_params* p, const nesf_io_fields* f, void* stream,
                         int part) {
    const char* who = "nesf_compute_sea_ice_ocean_fluxes";
    if (!p || !f) return fail(NESF_ERR_ARG, "%s: null argument", who);
    int r = check_grid(f->grid, 0, who);
    if (r) return r;
    if (f->dtype != NESF_F64 && f->dtype != NESF_F32) return fail(NESF_ERR_ARG, "%s: dtype %d", who, f->dtype);
    if (p->nz < 1) return fail(NESF_ERR_ARG, "%s: nz = %d", who, p->nz);
    if (p->nz > 1 && p->stride_k <= 0) return fail(NESF_ERR_ARG, "%s: stride_k must be > 0 for nz > 1", who);
    if (!(p->reference_latent_heat != 0) || !(p->dt > 0) || !(p->ocean_reference_density > 0))
        return fail(NESF_ERR_ARG, "%s: latent heat, dt and density must be nonzero/positive", who);
    const void* req[] = {f->T_oc, f->S_oc, f->dz, f->ice_salinity, f->ice_thickness, f->consolidation_thickness,
                         f->ice_concentration};
    for (const void* q : req)
        if (!q) return fail(NESF_ERR_ARG, "%s: a required array is NULL", who);
    if (p->conductive && p->formulation == 0 && !f->internal_temperature)
        return fail(NESF_ERR_ARG, "%s: conductive three-equation flux needs internal_temperature", who);
    DeviceGuard g(ctx ? ctx->device : 0);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = f->dtype == NESF_F64 ? launch_io(io_args<double>(f), *p, s, part)
                                         : launch_io(io_args<float>(f), *p, s, part);
    if (e != cudaSuccess) return cuda_fail(e, who);
    return NESF_OK;
}

extern "C" int nesf_compute_sea_ice_ocean_fluxes(nesf_context* ctx, const nesf_io_params* p, const nesf_io_fields* f,
                                                 void* stream) {
    return sea_ice_ocean(ctx, p, f, stream, 0);
}

extern "C" int nesf_compute_fractional_indices(const nesf_grid* g, const nesf_exchange_coords* c,
                                               const nesf_atmos_grid* a, double* fi, double* fj, void* stream) {
    const char* who = "nesf_compute_fractional_indices";
    if (!g || !c || !a || !fi || !fj) return fail(NESF_ERR_ARG, "%s: null argument", who);
    int r = check_grid(*g, 0, who);
    if (r) return r;
    if (!(a->dlon != 0) || !(a->dlat != 0)) return fail(NESF_ERR_ARG, "%s: zero atmosphere spacing", who);
    cudaError_t e = launch_frac(layout(*g), *c, *a, fi, fj, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, who);
    return NESF_OK;
}

extern "C" int nesf_interpolate_atmosphere_state(const nesf_interp_fields* f, void* stream) {
    const char* who = "nesf_interpolate_atmosphere_state";
    if (!f) return fail(NESF_ERR_ARG, "%s: null fields", who);
    int r = check_grid(f->grid, 1, who);
    if (r) return r;
    const nesf_atmos_grid& ag = f->atmos;
    if (ag.nx <= 0 || ag.ny <= 0 || ag.hx < 0 || ag.hy < 0 || ag.stride_j < (int64_t)ag.nx + 2 * ag.hx)
        return fail(NESF_ERR_ARG, "%s: atmosphere grid", who);
    if (!(ag.dlon != 0) || !(ag.dlat != 0)) return fail(NESF_ERR_ARG, "%s: zero atmosphere spacing", who);
    if (f->dtype != NESF_F64 && f->dtype != NESF_F32) return fail(NESF_ERR_ARG, "%s: dtype %d", who, f->dtype);
    if ((f->frac_i == nullptr) != (f->frac_j == nullptr))
        return fail(NESF_ERR_ARG, "%s: give both fractional index caches or neither", who);
    const void* src[9] = {f->u, f->v, f->T, f->q, f->p, f->rain, f->snow, f->sw_down, f->lw_down};
    void* dst[9] = {f->u_out, f->v_out, f->T_out, f->q_out, f->p_out, f->rain_out, f->snow_out, f->sw_out, f->lw_out};
    for (int k = 0; k < 5; k++)
        if (dst[k] && !src[k]) return fail(NESF_ERR_ARG, "%s: output %d requested without its input", who, k);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e;
    if (f->dtype == NESF_F64) {
        InterpArgs<double> a;
        a.L = layout(f->grid); a.coords = f->coords; a.atmos = ag; a.tn = f->time_weight;
        for (int k = 0; k < 9; k++) { a.src[k] = (const double*)src[k]; a.dst[k] = (double*)dst[k]; }
        a.frac_i = f->frac_i; a.frac_j = f->frac_j;
        e = launch_interp(a, s);
    } else {
        InterpArgs<float> a;
        a.L = layout(f->grid); a.coords = f->coords; a.atmos = ag; a.tn = f->time_weight;
        for (int k = 0; k < 9; k++) { a.src[k] = (const float*)src[k]; a.dst[k] = (float*)dst[k]; }
        a.frac_i = f->frac_i; a.frac_j = f->frac_j;
        e = launch_interp(a, s);
    }
    if (e != cudaSuccess) return cuda_fail(e, who);
    return NESF_OK;
}

template <class S>
static AsmArgs<S> asm_args(const nesf_assembly_fields* f, int with_rad) {
    AsmArgs<S> a;
    a.L = layout(f->grid);
    a.with_radiation = with_rad;
    AsmFields<S>& q = a.f;
    q.inactive = f->inactive;
    q.aleph = (const S*)f->ice_concentration; q.To = (const S*)f->ocean_surface_temperature;
    q.rain = (const S*)f->rain; q.snow = (const S*)f->snow; q.isnow = (const S*)f->intercepted_snow;
    q.land_fw = (const S*)f->land_freshwater;
    q.ao_QT = (const S*)f->ao_sensible; q.ao_Qv = (const S*)f->ao_latent; q.ao_Jv = (const S*)f->ao_water_vapor;
    q.ao_tx = (const S*)f->ao_x_momentum; q.ao_ty = (const S*)f->ao_y_momentum;
    q.ao_Ts = (const S*)f->ao_interface_temperature;
    q.io_Q = (const S*)f->io_interface_heat; q.io_Qf = (const S*)f->io_frazil_heat; q.io_Js = (const S*)f->io_salt;
    q.io_Jw = (const S*)f->io_freshwater; q.io_tx = (const S*)f->io_x_momentum; q.io_ty = (const S*)f->io_y_momentum;
    q.ai_QT = (const S*)f->ai_sensible; q.ai_Qv = (const S*)f->ai_latent; q.ai_tx = (const S*)f->ai_x_momentum;
    q.ai_ty = (const S*)f->ai_y_momentum; q.ai_Ts = (const S*)f->ai_interface_temperature;
    q.sw = (const S*)f->sw_down; q.lw = (const S*)f->lw_down;
    q.o_u = (S*)f->ocean_u; q.o_v = (S*)f->ocean_v; q.o_T = (S*)f->ocean_T; q.o_S = (S*)f->ocean_S;
    q.o_eta = (S*)f->ocean_eta; q.o_H = (S*)f->ocean_heat_content;
    q.i_top = (S*)f->ice_top_heat; q.i_snow = (S*)f->ice_top_snowfall; q.i_u = (S*)f->ice_top_u;
    q.i_v = (S*)f->ice_top_v; q.i_bottom = (S*)f->ice_bottom_heat;
    q.o_up_lw = (S*)f->ocean_upwelling_longwave; q.o_dn_lw = (S*)f->ocean_downwelling_longwave;
    q.o_dn_sw = (S*)f->ocean_downwelling_shortwave;
    q.i_up_lw = (S*)f->ice_upwelling_longwave; q.i_dn_lw = (S*)f->ice_downwelling_longwave;
    q.i_dn_sw = (S*)f->ice_downwelling_shortwave;
    return a;
}

static int check_assembly(const nesf_assembly_fields* f, int which, const char* who) {
    switch (which) {
    case 0:
        if (!f->ocean_surface_temperature || !f->ao_sensible || !f->ao_latent || !f->ao_water_vapor ||
            !f->ao_x_momentum || !f->ao_y_momentum)
            return fail(NESF_ERR_ARG, "%s: atmosphere-ocean fluxes and ocean temperature are required", who);
        break;
    case 1:
        if (!f->ice_concentration || !f->ai_sensible || !f->ai_latent || !f->ai_x_momentum || !f->ai_y_momentum)
            return fail(NESF_ERR_ARG, "%s: sea-ice concentration and atmosphere-sea-ice fluxes are required", who);
        break;
    case 2:
        if (!f->ao_interface_temperature || !f->sw_down || !f->lw_down || !f->ocean_T)
            return fail(NESF_ERR_ARG, "%s: T_s, radiation and ocean_T are required", who);
        break;
    default:
        if (!f->ai_interface_temperature || !f->sw_down || !f->lw_down || !f->ice_top_heat || !f->ice_concentration)
            return fail(NESF_ERR_ARG, "%s: T_s, radiation, concentration and top heat are required", who);
    }
    return NESF_OK;
}

// which: 0 ocean assembly, 1 sea-ice assembly, 2 / 3 their radiative add-ons. With
// `with_radiation` (which 0 or 1, the coupling step) the assembly kernel applies the
// add-on too, with the same operations in the same order as the separate pass (the
// assembled J_T / top heat flux rounded to the field's type, then the radiative part
// added), so the results are bit for bit those of the two calls.
static int run_assembly(const nesf_assembly_params* p, const nesf_assembly_fields* f, int which, void* stream,
                        const char* who, int with_radiation = 0) {
    if (!p || !f) return fail(NESF_ERR_ARG, "%s: null argument", who);
    int r = check_grid(f->grid, 1, who);
    if (r) return r;
    if (f->dtype != NESF_F64 && f->dtype != NESF_F32) return fail(NESF_ERR_ARG, "%s: dtype %d", who, f->dtype);
    if (!(p->ocean_reference_density > 0) || !(p->ocean_heat_capacity > 0))
        return fail(NESF_ERR_ARG, "%s: density and heat capacity must be positive", who);
    if ((r = check_assembly(f, which, who))) return r;
    if (with_radiation && (r = check_assembly(f, which + 2, who))) return r;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = f->dtype == NESF_F64 ? launch_assemble(asm_args<double>(f, with_radiation), *p, which, s)
                                         : launch_assemble(asm_args<float>(f, with_radiation), *p, which, s);
    if (e != cudaSuccess) return cuda_fail(e, who);
    return NESF_OK;
}

extern "C" int nesf_assemble_net_ocean_fluxes(const nesf_assembly_params* p, const nesf_assembly_fields* f,
                                              void* stream) {
    return run_assembly(p, f, 0, stream, "nesf_assemble_net_ocean_fluxes");
}
extern "C" int nesf_assemble_net_sea_ice_fluxes(const nesf_assembly_params* p, const nesf_assembly_fields* f,
                                                void* stream) {
    return run_assembly(p, f, 1, stream, "nesf_assemble_net_sea_ice_fluxes");
}
extern "C" int nesf_apply_air_sea_radiative_fluxes(const nesf_assembly_params* p, const nesf_assembly_fields* f,
                                                   void* stream) {
    return run_assembly(p, f, 2, stream, "nesf_apply_air_sea_radiative_fluxes");
}
extern "C" int nesf_apply_air_sea_ice_radiative_fluxes(const nesf_assembly_params* p, const nesf_assembly_fields* f,
                                                       void* stream) {
    return run_assembly(p, f, 3, stream, "nesf_apply_air_sea_ice_radiative_fluxes");
}

template <class S>
static LandArgs<S> land_args(const nesf_land_flux_fields* f) {
    LandArgs<S> a;
    a.L = layout(f->grid);
    a.inactive = f->inactive;
    a.rain = (const S*)f->rain;
    a.QT = (const S*)f->al_sensible; a.Qv = (const S*)f->al_latent; a.Jv = (const S*)f->al_water_vapor;
    a.Ts = (const S*)f->al_interface_temperature;
    a.sw = (const S*)f->sw_down; a.lw = (const S*)f->lw_down;
    a.Es = (S*)f->surface_energy_flux; a.P = (S*)f->precipitation; a.E = (S*)f->evaporation;
    a.Jvo = (S*)f->vapor_flux; a.Pl = (S*)f->liquid_precipitation_flux;
    a.up_lw = (S*)f->upwelling_longwave; a.dn_lw = (S*)f->downwelling_longwave;
    a.dn_sw = (S*)f->downwelling_shortwave;
    return a;
}

static int run_land(const nesf_land_radiation_params* p, const nesf_land_flux_fields* f, bool radiation, void* stream,
                    const char* who) {
    if (!f || (radiation && !p)) return fail(NESF_ERR_ARG, "%s: null argument", who);
    int r = check_grid(f->grid, 0, who);
    if (r) return r;
    if (f->dtype != NESF_F64 && f->dtype != NESF_F32) return fail(NESF_ERR_ARG, "%s: dtype %d", who, f->dtype);
    if (radiation) {
        if (!f->al_interface_temperature || !f->sw_down || !f->lw_down || !f->surface_energy_flux)
            return fail(NESF_ERR_ARG, "%s: T_s, radiation and surface_energy_flux are required", who);
    } else if (!f->al_sensible || !f->al_latent || !f->al_water_vapor) {
        return fail(NESF_ERR_ARG, "%s: the atmosphere-land fluxes are required", who);
    }
    nesf_land_radiation_params q = {};
    if (p) q = *p;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = f->dtype == NESF_F64 ? launch_land(land_args<double>(f), q, radiation, s)
                                         : launch_land(land_args<float>(f), q, radiation, s);
    if (e != cudaSuccess) return cuda_fail(e, who);
    return NESF_OK;
}

extern "C" int nesf_assemble_net_land_fluxes(const nesf_land_flux_fields* f, void* stream) {
    return run_land(nullptr, f, false, stream, "nesf_assemble_net_land_fluxes");
}
extern "C" int nesf_apply_air_land_radiative_fluxes(const nesf_land_radiation_params* p, const nesf_land_flux_fields* f,
                                                    void* stream) {
    return run_land(p, f, true, stream, "nesf_apply_air_land_radiative_fluxes");
}

// ------------------------------------------------ allocation-free variant
// Some callers cannot allocate device memory when they run the flux step: a host
// model whose memory manager has reserved the whole device (the pooling allocators
// of CUDA.jl or PyTorch can hold every free byte, so a cudaMalloc inside the call
// would fail or force the pool to release memory), or a caller with a latency
// budget that must not enter the driver's allocator. For them,
// nesf_compute_atmosphere_ocean_fluxes_noalloc runs the atmosphere-ocean solve
// without allocating anything: its scratch -- the compacted work list, the queues
// of cells to replay and to polish, and their counters -- is this file-scope array:
// 64 counters (256 B) + three lists of NESF_NOALLOC_MAX_CELLS uint32 entries, 24 MiB
// + 256 B in all. Under lazy module loading (the CUDA default) a device holds the
// array from the moment this file's module is loaded on it, which
// nesf_noalloc_prepare does; from then until the process exits.
#define NESF_NOALLOC_MAX_CELLS (1 << 21)
static __device__ __align__(256) uint32_t g_noalloc_scratch[64 + 3 * (size_t)NESF_NOALLOC_MAX_CELLS];

static uint32_t* g_noalloc_ptr[64];   // device address of the array, per prepared device
static std::mutex g_noalloc_lock;

// Set-up, once per device, with that device current: the array's device address
// (in host code the symbol names a host-side stand-in, not device memory, so only
// this address may be handed to a kernel), and every kernel the entry point can
// launch loaded, so that its calls load no module (loading one allocates).
extern "C" int nesf_noalloc_prepare(int32_t device) {
    const char* who = "nesf_noalloc_prepare";
    int n = 0;
    NESF_CUDA(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n || device >= 64) return fail(NESF_ERR_ARG, "%s: device %d of %d", who, device, n);
    std::lock_guard<std::mutex> lk(g_noalloc_lock);
    if (g_noalloc_ptr[device]) return NESF_OK;
    DeviceGuard g(device);
    if (!g.ok) return fail(NESF_ERR_CUDA, "%s: cannot make device %d current", who, device);
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(scratch)");
    if ((e = preload_ao_kernels((const AOArgs<double>*)nullptr)) != cudaSuccess ||
        (e = preload_ao_kernels((const AOArgs<float>*)nullptr)) != cudaSuccess)
        return cuda_fail(e, "nesf_noalloc_prepare: loading the solve kernels");
    g_noalloc_ptr[device] = (uint32_t*)p;
    return NESF_OK;
}

extern "C" int nesf_compute_atmosphere_ocean_fluxes_noalloc(const nesf_interface_params* params,
                                                            const nesf_ao_fields* f, const nesf_solver_options* opts,
                                                            void* stream) {
    const char* who = "nesf_compute_atmosphere_ocean_fluxes_noalloc";
    int r = check_params(params, who);
    if (r) return r;
    if ((r = check_ao_fields(f, params, who))) return r;
    nesf_solver_options o = options_or_default(opts);
    if ((r = check_options(o, who))) return r;
    if (o.warm_start) return fail(NESF_ERR_ARG, "%s: no warm start (its buffers would be allocated)", who);
    int64_t ring = (int64_t)(f->grid.nx + 2) * (f->grid.ny + 2);
    if (ring > NESF_NOALLOC_MAX_CELLS)
        return fail(NESF_ERR_CAPACITY,
                    "%s: %lld cells (halo ring included) exceed the fixed scratch of %d cells; "
                    "use nesf_compute_atmosphere_ocean_fluxes", who, (long long)ring, NESF_NOALLOC_MAX_CELLS);
    int dev = 0;
    NESF_CUDA(cudaGetDevice(&dev));
    uint32_t* base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_noalloc_lock);
        if (dev >= 0 && dev < 64) base = g_noalloc_ptr[dev];
    }
    if (!base) return fail(NESF_ERR_ARG, "%s: device %d not prepared (call nesf_noalloc_prepare(%d) at set-up)", who,
                            dev, dev);
    // counters: base[0..1] the work list's counts (unstable, stable); base[2..6] the
    // queue counters rq.count[0..4] (replays, polishes, the sea-ice solve's polish and
    // calm replays (unused here), pass 1's fetch counter); the launch clears the counters
    // a precision uses before its first pass reads them
    WorkList wl{base + 64, base, ring};
    ReplayQueue rq{base + 64 + NESF_NOALLOC_MAX_CELLS, base + 2, NESF_NOALLOC_MAX_CELLS, nullptr};
    DevIface<double> P64 = make_dev_iface<double>(*params);
    DevIface<float> P32 = make_dev_iface<float>(*params);
    bool skin = params->temperature_formulation != NESF_BULK_TEMPERATURE;
    SolveOpts so = solve_opts(o);
    const DevIface<df> Pdf = make_dev_iface<df>(*params);
    so.pdf = &Pdf;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = f->dtype == NESF_F64
                        ? launch_ao(ao_args<double>(f, 0), P64, P32, nullptr, nullptr, 1, o.precision, skin, so, wl,
                                    rq, WarmStart{}, nullptr, s)
                        : launch_ao(ao_args<float>(f, 0), P64, P32, nullptr, nullptr, 1, o.precision, skin, so, wl,
                                    rq, WarmStart{}, nullptr, s);
    if (e != cudaSuccess) return cuda_fail(e, who);
    return NESF_OK;
}

// ------------------------------------------------ double-float check
namespace nesf {
cudaError_t launch_df_check(const double* x, const double* y, double* out, int64_t n, int op, cudaStream_t s);
}

extern "C" int nesf_double_float_check(const double* x, const double* y, double* out, int64_t n, int32_t op,
                                       void* stream) {
    const char* who = "nesf_double_float_check";
    if (op < NESF_DF_ADD || op > NESF_DF_ATAN) return fail(NESF_ERR_ARG, "%s: operation %d", who, op);
    const bool binary = op == NESF_DF_ADD || op == NESF_DF_SUB || op == NESF_DF_MUL || op == NESF_DF_DIV ||
                        op == NESF_DF_POW;
    if (n < 0 || n > ((int64_t)1 << 31)) return fail(NESF_ERR_ARG, "%s: n = %lld", who, (long long)n);
    if (n > 0 && (!x || !out || (binary && !y))) return fail(NESF_ERR_ARG, "%s: null array", who);
    if (n == 0) return NESF_OK;
    cudaError_t e = nesf::launch_df_check(x, binary ? y : nullptr, out, n, op, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, who);
    return NESF_OK;
}

// ---------------------------------------------------- tensor-core check
namespace nesf {
cudaError_t launch_tc_selftest(const void* A, const void* B, float* D, int which, unsigned int* status,
                               cudaStream_t s);
}

extern "C" int nesf_mlp_selftest(const void* a, const void* b, float* d, int32_t which, void* stream) {
    const char* who = "nesf_mlp_selftest";
    if (!a || !b || !d) return fail(NESF_ERR_ARG, "%s: null argument", who);
    if (which < 0 || which > 3) return fail(NESF_ERR_ARG, "%s: which = %d", who, which);
    unsigned int* st = nullptr;
    NESF_CUDA(cudaMalloc(&st, sizeof(unsigned int)));
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(st, 0, sizeof(unsigned int), s);
    if (e == cudaSuccess) e = launch_tc_selftest(a, b, d, which, st, s);
    unsigned int h = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, st, sizeof h, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(st);
    if (e != cudaSuccess) return cuda_fail(e, who);
    if (h) return fail(NESF_ERR_TIMEOUT, "%s: the MMA did not complete", who);
    return NESF_OK;
}

// ------------------------------------------------------ warm-start network
namespace nesf {
cudaError_t mlp_init(void* blob, uint64_t seed, cudaStream_t s);
cudaError_t mlp_fit_normalization(void* blob, const float* x, const float* t, int64_t n, cudaStream_t s);
cudaError_t mlp_adam(void* blob, float lr, float beta1, float beta2, float eps, cudaStream_t s);
size_t mlp_blob_bytes();
size_t mlp_loss_offset();
}

static int sm_count() {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

extern "C" int64_t nesf_mlp_bytes(void) { return (int64_t)mlp_blob_bytes(); }

extern "C" int nesf_mlp_init(void* mlp, uint64_t seed, void* stream) {
    if (!mlp) return fail(NESF_ERR_ARG, "nesf_mlp_init: null blob");
    cudaError_t e = mlp_init(mlp, seed, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "nesf_mlp_init");
    return NESF_OK;
}

extern "C" int nesf_mlp_fit_normalization(void* mlp, const float* x, const float* t, int64_t n, void* stream) {
    if (!mlp || !x || !t || n <= 0) return fail(NESF_ERR_ARG, "nesf_mlp_fit_normalization: bad argument");
    cudaError_t e = mlp_fit_normalization(mlp, x, t, n, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "nesf_mlp_fit_normalization");
    return NESF_OK;
}

// The tile pass reads each sample's 8 features as two 16-byte vectors.
static bool features_aligned(const float* x) { return ((uintptr_t)x & 15u) == 0; }

extern "C" int nesf_mlp_gradient(void* mlp, const float* x, const float* t, int64_t n, void* stream) {
    if (!mlp || !x || !t || n <= 0) return fail(NESF_ERR_ARG, "nesf_mlp_gradient: bad argument");
    if (!features_aligned(x)) return fail(NESF_ERR_ARG, "nesf_mlp_gradient: features not 16-byte aligned");
    int64_t tiles = (n + 127) / 128;
    int grid = (int)(tiles < sm_count() ? tiles : sm_count());
    cudaError_t e = mlp_pass(mlp, x, t, nullptr, n, nullptr, 0, grid, false, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "nesf_mlp_gradient");
    return NESF_OK;
}

extern "C" int nesf_mlp_train(void* mlp, const float* x, const float* t, int64_t n, const nesf_mlp_train_options* o,
                              float* loss, void* stream) {
    const char* who = "nesf_mlp_train";
    if (!mlp || !x || !t || !o || n <= 0) return fail(NESF_ERR_ARG, "%s: bad argument", who);
    if (!features_aligned(x)) return fail(NESF_ERR_ARG, "%s: features not 16-byte aligned", who);
    if (o->batch <= 0 || o->batch % 128 != 0) return fail(NESF_ERR_ARG, "%s: batch %d not a multiple of 128", who, o->batch);
    if (o->epochs <= 0 || !(o->learning_rate > 0)) return fail(NESF_ERR_ARG, "%s: epochs / learning rate", who);
    cudaStream_t s = (cudaStream_t)stream;
    const int sms = sm_count();
    float* loss_dev = (float*)((char*)mlp + mlp_loss_offset());
    for (int ep = 0; ep < o->epochs; ep++) {
        cudaError_t e = cudaMemsetAsync(loss_dev, 0, 2 * sizeof(float), s);
        for (int64_t b0 = 0; e == cudaSuccess && b0 < n; b0 += o->batch) {
            int64_t nb = n - b0 < o->batch ? n - b0 : o->batch;
            int64_t tiles = (nb + 127) / 128;
            int grid = (int)(tiles < sms ? tiles : sms);
            e = mlp_pass(mlp, x + b0 * 8, t + b0 * 4, nullptr, nb, nullptr, 0, grid, false, s);
            if (e == cudaSuccess) e = mlp_adam(mlp, o->learning_rate, o->beta1, o->beta2, o->eps, s);
        }
        if (e == cudaSuccess && loss) {
            float h[2] = {0.0f, 0.0f};
            e = cudaMemcpyAsync(h, loss_dev, sizeof h, cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            loss[ep] = h[1] > 0 ? h[0] / h[1] : 0.0f;
        }
        if (e != cudaSuccess) return cuda_fail(e, who);
    }
    return NESF_OK;
}

extern "C" int nesf_mlp_infer(void* mlp, const float* x, int64_t n, float* out, void* stream) {
    if (!mlp || !x || !out || n <= 0) return fail(NESF_ERR_ARG, "nesf_mlp_infer: bad argument");
    if (!features_aligned(x)) return fail(NESF_ERR_ARG, "nesf_mlp_infer: features not 16-byte aligned");
    int64_t tiles = (n + 127) / 128;
    int grid = (int)(tiles < sm_count() ? tiles : sm_count());
    cudaError_t e = mlp_pass(mlp, x, nullptr, out, n, nullptr, 0, grid, false, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "nesf_mlp_infer");
    return NESF_OK;
}

extern "C" int nesf_mlp_ao_samples(const nesf_interface_params* params, const nesf_ao_fields* f, float* feat,
                                   float* targ, void* stream) {
    const char* who = "nesf_mlp_ao_samples";
    int r = check_params(params, who);
    if (r) return r;
    if ((r = check_ao_fields(f, params, who))) return r;
    if (!feat) return fail(NESF_ERR_ARG, "%s: null features", who);
    if (targ && (!f->friction_velocity || !f->temperature_scale || !f->water_vapor_scale))
        return fail(NESF_ERR_ARG, "%s: targets need the solved u*, theta*, q* fields", who);
    DevIface<float> P32 = make_dev_iface<float>(*params);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = f->dtype == NESF_F64 ? launch_ao_samples(ao_args<double>(f, 0), P32, feat, targ, s)
                                         : launch_ao_samples(ao_args<float>(f, 0), P32, feat, targ, s);
    if (e != cudaSuccess) return cuda_fail(e, who);
    return NESF_OK;
}

// ------------------------------------------------------------ area integrals
extern "C" int nesf_area_integrals(nesf_context* ctx, const nesf_integral_fields* f, double* result, void* stream) {
    const char* who = "nesf_area_integrals";
    if (!f || !result) return fail(NESF_ERR_ARG, "%s: null argument", who);
    int r = check_grid(f->grid, 0, who);
    if (r) return r;
    if (f->dtype != NESF_F64 && f->dtype != NESF_F32) return fail(NESF_ERR_ARG, "%s: dtype %d", who, f->dtype);
    if (f->n < 1 || f->n > NESF_MAX_INTEGRALS) return fail(NESF_ERR_ARG, "%s: n = %d", who, f->n);
    for (int k = 0; k < f->n; k++)
        if (!f->field[k]) return fail(NESF_ERR_ARG, "%s: field %d is NULL", who, k);
    if (f->area && f->row_area) return fail(NESF_ERR_ARG, "%s: give area or row_area, not both", who);
    if ((r = context_or_default(&ctx))) return r;
    std::lock_guard<std::mutex> lk(ctx->lock);
    DeviceGuard g(ctx->device);
    cudaError_t e = launch_integrals(*f, ctx->d_partials, kIntegralBlocks, result, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, who);
    return NESF_OK;
}

// ------------------------------------------------------------ coupling step
// Scratch for the solves of a step, sized before any capture (growing it
// synchronises the device, which a stream capture forbids).
static int size_scratch(nesf_context* ctx, int64_t cells, const nesf_solver_options* opts, bool sea_ice = false) {
    std::lock_guard<std::mutex> lk(ctx->lock);
    DeviceGuard g(ctx->device);
    ReplayQueue rq;
    WorkList wl;
    WarmStart ws;
    int r = replay_queue(ctx, cells, &rq, sea_ice);
    if (r == NESF_OK) r = work_list(ctx, cells, 1, &wl);
    if (r == NESF_OK) r = warm_buffers(ctx, options_or_default(opts), cells, &ws);
    return r;
}

// The second lane of the coupling step: a scratch set for the sea-ice solve, a
// stream and three events (created once; never during a stream capture).
static int coupling_lane(nesf_context* ctx) {
    if (ctx->aux) return NESF_OK;
    DeviceGuard g(ctx->device);
    int r = nesf_context_create(ctx->device, &ctx->aux);
    if (r) return r;
    NESF_CUDA(cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking));
    NESF_CUDA(cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
    NESF_CUDA(cudaEventCreateWithFlags(&ctx->ev_ice, cudaEventDisableTiming));
    NESF_CUDA(cudaEventCreateWithFlags(&ctx->ev_ocean, cudaEventDisableTiming));
    NESF_CUDA(cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming));
    return NESF_OK;
}

static int coupling_scratch(nesf_context* ctx, const nesf_coupling_step_args* a, const nesf_solver_options* opts) {
    int r = size_scratch(ctx, (int64_t)(a->ao->grid.nx + 2) * (a->ao->grid.ny + 2), opts);
    if (r == NESF_OK) r = tail_lane(ctx);   // the ocean solve's replay lane
    if (r == NESF_OK && a->ai_params && a->ai) {
        if ((r = coupling_lane(ctx))) return r;
        if ((r = tail_lane(ctx->aux))) return r;
        r = size_scratch(ctx->aux, (int64_t)(a->ai->grid.nx + 2) * (a->ai->grid.ny + 2), opts, true);
    }
    return r;
}

extern "C" int nesf_coupling_step(nesf_context* ctx, const nesf_coupling_step_args* a,
                                  const nesf_solver_options* opts, void* stream) {
    const char* who = "nesf_coupling_step";
    if (!a || !a->ao_params || !a->ao) return fail(NESF_ERR_ARG, "%s: the atmosphere-ocean interface is required", who);
    if (a->radiation && !a->assembly_params) return fail(NESF_ERR_ARG, "%s: radiation needs the assembly", who);
    if (a->assembly_params && !a->assembly) return fail(NESF_ERR_ARG, "%s: assembly parameters without fields", who);
    if ((a->ai_params == nullptr) != (a->ai == nullptr) || (a->io_params == nullptr) != (a->io == nullptr))
        return fail(NESF_ERR_ARG, "%s: give the parameters and the fields of an interface together", who);
    int r = context_or_default(&ctx);
    if (r) return r;
    const bool ice = a->ai_params != nullptr;
    // update_state! order (time_step_earth_system_model.jl:50-80), with the two interface
    // solves on two lanes: the sea-ice solve runs first on the side stream; the ocean solve
    // starts when its pass 1 is done and overlaps its packed polish and replay passes, which
    // are latency-bound (few cells, long FP64 iterations). The sea-ice-ocean fluxes read
    // only the ocean and ice state, so they run on the main lane beside the sea-ice pass 1;
    // their frazil adjustment of the ocean temperature, which both solves read, waits for
    // both (the same state as update_state!'s order).
    // The context's tuning may put the sea-ice solve in line (one lane) and the
    // sea-ice-ocean fluxes after the solves; the outputs are the same.
    cudaStream_t s = (cudaStream_t)stream;
    const Tracer* tr = tracer_of(ctx);
    if (tr) {
        ctx->trace->n = 0;
        trace_mark(tr, "step", s);
    }
    if (a->interp && (r = nesf_interpolate_atmosphere_state(a->interp, stream))) return r;
    if (a->interp) trace_mark(tr, "interpolate", s);
    const bool io_split = ice && a->io_params && ctx->tuning.io_overlap;
    const bool lanes = ice && ctx->tuning.two_lanes;
    // early_ocean_classify 2: the sea-ice lane is enqueued from inside the ocean solve, once
    // the ocean's classify pass and inference are, and its pass 1 waits for them (ev_ocean).
    // 3: the ocean solve is enqueued from inside the sea-ice solve, after its pass 1, waits for
    // that pass, and the sea-ice polish pass waits for the ocean's inference (ev_ocean): the
    // ocean's classify and inference run alone after the sea-ice pass 1, the sea-ice polish
    // beside the ocean's pass 1
    const bool ocean_first = lanes && ctx->tuning.early_ocean_classify == 2;
    const bool ice_polish_later = lanes && ctx->tuning.early_ocean_classify == 3;
    struct IceLane {
        nesf_context* ctx;
        const nesf_coupling_step_args* a;
        const nesf_solver_options* opts;
    } lane{ctx, a, opts};
    MidHook mid{nullptr, nullptr, NESF_OK, nullptr, nullptr};
    if (ice) {
        if ((r = coupling_lane(ctx))) return r;
        ctx->aux->tuning = ctx->tuning;
        ctx->aux->trace = ctx->trace;   // one timeline for both lanes
        DeviceGuard g(ctx->device);
        if (lanes) {
            NESF_CUDA(cudaEventRecord(ctx->ev_fork, s));
            NESF_CUDA(cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0));
            if (!ocean_first && !ice_polish_later) {
                if ((r = sea_ice_fluxes(ctx->aux, a->ai_params, a->ai, opts, nullptr, ctx->side, ctx->ev_ice)))
                    return r;
                NESF_CUDA(cudaEventRecord(ctx->ev_join, ctx->side));
            }
        }
        if (io_split && (r = sea_ice_ocean(ctx, a->io_params, a->io, stream, 1))) return r;
        if (io_split) trace_mark(tr, "sea_ice_ocean_fluxes", s);
        if (ice_polish_later) {
            // the ocean solve on the main stream (after the sea-ice pass 1), enqueued from the
            // sea-ice launch once its pass 1 is
            struct OceanLane {
                nesf_context* ctx;
                const nesf_coupling_step_args* a;
                const nesf_solver_options* opts;
                cudaStream_t s;
            } ol{ctx, a, opts, s};
            MidHook om{nullptr, nullptr, NESF_OK, ctx->ev_ocean, nullptr};
            struct Both { OceanLane* ol; MidHook* om; } both{&ol, &om};
            MidHook im{nullptr, &both, NESF_OK, nullptr, ctx->ev_ocean};
            im.fn = [](void* p) -> int {
                Both* b = (Both*)p;
                const cudaError_t e = cudaStreamWaitEvent(b->ol->s, b->ol->ctx->ev_ice, 0);
                if (e != cudaSuccess) return cuda_fail(e, "nesf_coupling_step");
                const int q = ocean_fluxes(b->ol->ctx, b->ol->a->ao_params, b->ol->a->ao, b->ol->opts, nullptr,
                                           (void*)b->ol->s, nullptr, b->om);
                return b->om->status ? b->om->status : q;
            };
            r = sea_ice_fluxes(ctx->aux, a->ai_params, a->ai, opts, nullptr, ctx->side, ctx->ev_ice, nullptr, &im);
            if (im.status) return im.status;
            if (r) return r;
            NESF_CUDA(cudaEventRecord(ctx->ev_join, ctx->side));
        }
        if (lanes && !ctx->tuning.early_ocean_classify) NESF_CUDA(cudaStreamWaitEvent(s, ctx->ev_ice, 0));
        else if (!lanes && (r = sea_ice_fluxes(ctx->aux, a->ai_params, a->ai, opts, nullptr, s, nullptr))) return r;
        if (ocean_first) {
            mid.ready = ctx->ev_ocean;
            mid.arg = &lane;
            mid.fn = [](void* p) -> int {
                IceLane* l = (IceLane*)p;
                int q = sea_ice_fluxes(l->ctx->aux, l->a->ai_params, l->a->ai, l->opts, nullptr, l->ctx->side,
                                       l->ctx->ev_ice, l->ctx->ev_ocean);
                if (q) return q;
                const cudaError_t e = cudaEventRecord(l->ctx->ev_join, l->ctx->side);
                return e == cudaSuccess ? NESF_OK : cuda_fail(e, "nesf_coupling_step");
            };
        }
    }
    // with early_ocean_classify 1 the ocean's classify pass and warm-start inference run beside
    // the sea-ice pass 1, with 2 before it; either way the ocean's pass 1 waits for the sea-ice
    // pass 1
    cudaEvent_t before_pass1 = lanes && ctx->tuning.early_ocean_classify ? ctx->ev_ice : nullptr;
    if (!ice_polish_later) {
        r = ocean_fluxes(ctx, a->ao_params, a->ao, opts, nullptr, stream, before_pass1, ocean_first ? &mid : nullptr);
        if (mid.status) return mid.status;
        if (r) return r;
    }
    if (lanes) {
        DeviceGuard g(ctx->device);
        NESF_CUDA(cudaStreamWaitEvent(s, ctx->ev_join, 0));
    }
    if (a->io_params && (r = sea_ice_ocean(ctx, a->io_params, a->io, stream, io_split ? 2 : 0))) return r;
    if (a->io_params) trace_mark(tr, io_split ? "frazil_adjustment" : "sea_ice_ocean_fluxes", s);
    if (a->assembly_params) {
        // the radiative add-ons inside the assembly kernels (bit for bit the separate passes)
        const int rad = a->radiation ? 1 : 0;
        if ((r = run_assembly(a->assembly_params, a->assembly, 0, stream, "nesf_coupling_step (ocean assembly)", rad)))
            return r;
        if (ice && (r = run_assembly(a->assembly_params, a->assembly, 1, stream,
                                     "nesf_coupling_step (sea-ice assembly)", rad)))
            return r;
        trace_mark(tr, "assembly", s);
    }
    return NESF_OK;
}

struct nesf_graph {
    int device;
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    cudaGraphNode_t interp_node;           // null when the step has no interpolation
    cudaKernelNodeParams interp_params;    // its launch configuration
    alignas(16) unsigned char interp_args[sizeof(InterpArgs<double>)];   // its argument, time weight updated
    bool interp_fp64;
};

extern "C" int nesf_graph_capture(nesf_context* ctx, const nesf_coupling_step_args* a,
                                  const nesf_solver_options* opts, nesf_graph** out) {
    const char* who = "nesf_graph_capture";
    if (!out) return fail(NESF_ERR_ARG, "%s: null output pointer", who);
    *out = nullptr;
    if (!a || !a->ao_params || !a->ao) return fail(NESF_ERR_ARG, "%s: the atmosphere-ocean interface is required", who);
    int r = context_or_default(&ctx);
    if (r) return r;
    if ((r = coupling_scratch(ctx, a, opts))) return r;
    DeviceGuard g(ctx->device);
    nesf_graph* G = new (std::nothrow) nesf_graph();
    if (!G) return fail(NESF_ERR_ARG, "%s: out of host memory", who);
    G->device = ctx->device;
    cudaStream_t cs = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        if (cs) cudaStreamDestroy(cs);
        delete G;
        return cuda_fail(e, "nesf_graph_capture: begin");
    }
    r = nesf_coupling_step(ctx, a, opts, cs);
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(cs, &graph);
    cudaStreamDestroy(cs);
    if (r != NESF_OK || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        delete G;
        return r != NESF_OK ? r : cuda_fail(e, "nesf_graph_capture: end");
    }
    G->graph = graph;
    // the interpolation node, whose time weight changes every step
    if (a->interp) {
        G->interp_fp64 = a->interp->dtype == NESF_F64;
        size_t n = 0;
        e = cudaGraphGetNodes(graph, nullptr, &n);
        cudaGraphNode_t nodes[256];
        if (e == cudaSuccess && n <= 256) e = cudaGraphGetNodes(graph, nodes, &n);
        for (size_t k = 0; e == cudaSuccess && k < n && k < 256; k++) {
            cudaGraphNodeType t;
            if (cudaGraphNodeGetType(nodes[k], &t) != cudaSuccess || t != cudaGraphNodeTypeKernel) continue;
            cudaKernelNodeParams kp;
            if (cudaGraphKernelNodeGetParams(nodes[k], &kp) != cudaSuccess || !is_interp_kernel(kp.func, G->interp_fp64))
                continue;
            G->interp_node = nodes[k];
            G->interp_params = kp;
            memcpy(G->interp_args, kp.kernelParams[0],
                   G->interp_fp64 ? sizeof(InterpArgs<double>) : sizeof(InterpArgs<float>));
        }
        if (e == cudaSuccess && !G->interp_node) e = cudaErrorInvalidValue;
        if (e != cudaSuccess) {
            cudaGraphDestroy(graph);
            delete G;
            return cuda_fail(e, "nesf_graph_capture: interpolation node");
        }
    }
    e = cudaGraphInstantiate(&G->exec, graph, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        delete G;
        return cuda_fail(e, "nesf_graph_capture: instantiate");
    }
    *out = G;
    return NESF_OK;
}

extern "C" int nesf_graph_set_time_weight(nesf_graph* G, double tn) {
    if (!G) return fail(NESF_ERR_ARG, "nesf_graph_set_time_weight: null graph");
    if (!G->interp_node) return fail(NESF_ERR_ARG, "nesf_graph_set_time_weight: the graph has no interpolation");
    if (!(tn >= 0.0 && tn <= 1.0)) return fail(NESF_ERR_ARG, "nesf_graph_set_time_weight: weight %g", tn);
    DeviceGuard g(G->device);
    if (G->interp_fp64) ((InterpArgs<double>*)G->interp_args)->tn = tn;
    else ((InterpArgs<float>*)G->interp_args)->tn = tn;
    void* args[1] = {G->interp_args};
    cudaKernelNodeParams kp = G->interp_params;
    kp.kernelParams = args;
    kp.extra = nullptr;
    NESF_CUDA(cudaGraphExecKernelNodeSetParams(G->exec, G->interp_node, &kp));
    return NESF_OK;
}

// The snapshot pair a captured step's interpolation reads, for a forcing window that moves
// the pair between device slots: per variable the first snapshot (NULL keeps the captured
// pointer), the stride to the second one and the pair's time weight.
template <class S>
static int set_forcing_args(InterpArgs<S>* a, const void* const* src, int64_t stride_t, double tn) {
    for (int n = 0; n < 9; n++) {
        if (!src || !src[n]) continue;
        if (!a->src[n])
            return fail(NESF_ERR_ARG, "nesf_graph_set_forcing: variable %d was not interpolated at capture", n);
        if (((uintptr_t)src[n]) % sizeof(S))
            return fail(NESF_ERR_ARG, "nesf_graph_set_forcing: variable %d is not aligned to its type", n);
    }
    for (int n = 0; n < 9; n++)
        if (src && src[n]) a->src[n] = (const S*)src[n];
    a->atmos.stride_t = stride_t;
    a->tn = tn;
    return NESF_OK;
}

extern "C" int nesf_graph_set_forcing(nesf_graph* G, const void* const* src, int64_t stride_t, double tn) {
    if (!G) return fail(NESF_ERR_ARG, "nesf_graph_set_forcing: null graph");
    if (!G->interp_node) return fail(NESF_ERR_ARG, "nesf_graph_set_forcing: the graph has no interpolation");
    if (!(tn >= 0.0 && tn <= 1.0)) return fail(NESF_ERR_ARG, "nesf_graph_set_forcing: weight %g", tn);
    DeviceGuard g(G->device);
    int r = G->interp_fp64 ? set_forcing_args((InterpArgs<double>*)G->interp_args, src, stride_t, tn)
                           : set_forcing_args((InterpArgs<float>*)G->interp_args, src, stride_t, tn);
    if (r) return r;
    void* args[1] = {G->interp_args};
    cudaKernelNodeParams kp = G->interp_params;
    kp.kernelParams = args;
    kp.extra = nullptr;
    NESF_CUDA(cudaGraphExecKernelNodeSetParams(G->exec, G->interp_node, &kp));
    return NESF_OK;
}

extern "C" int nesf_graph_launch(nesf_graph* G, void* stream) {
    if (!G) return fail(NESF_ERR_ARG, "nesf_graph_launch: null graph");
    DeviceGuard g(G->device);
    NESF_CUDA(cudaGraphLaunch(G->exec, (cudaStream_t)stream));
    return NESF_OK;
}

extern "C" int nesf_graph_destroy(nesf_graph* G) {
    if (!G) return NESF_OK;
    DeviceGuard g(G->device);
    if (G->exec) cudaGraphExecDestroy(G->exec);
    if (G->graph) cudaGraphDestroy(G->graph);
    delete G;
    return NESF_OK;
}

// ---------------------------------------------------------------- tracing
extern "C" int nesf_trace_enable(nesf_context* ctx, int32_t on) {
    int r = context_or_default(&ctx);
    if (r) return r;
    std::lock_guard<std::mutex> lk(ctx->lock);
    if (on && !ctx->trace) {
        DeviceGuard g(ctx->device);
        TraceBuf* t = new (std::nothrow) TraceBuf();
        if (!t) return fail(NESF_ERR_ARG, "nesf_trace_enable: out of host memory");
        for (int i = 0; i < NESF_TRACE_MAX; i++) {
            cudaError_t e = cudaEventCreate(&t->ev[i]);
            if (e != cudaSuccess) {
                for (int j = 0; j < i; j++) cudaEventDestroy(t->ev[j]);
                delete t;
                return cuda_fail(e, "nesf_trace_enable");
            }
        }
        t->hook = Tracer{trace_record, t};
        ctx->trace = t;
        ctx->trace_owned = true;
    }
    if (ctx->trace) ctx->trace->on = on != 0;
    return NESF_OK;
}

extern "C" int nesf_trace_read(nesf_context* ctx, nesf_trace_entry* out, int32_t max, int32_t* count) {
    if (!out || !count || max < 0) return fail(NESF_ERR_ARG, "nesf_trace_read: null output or max < 0");
    int r = context_or_default(&ctx);
    if (r) return r;
    std::lock_guard<std::mutex> lk(ctx->lock);
    *count = 0;
    TraceBuf* t = ctx->trace;
    if (!t || t->n == 0) return NESF_OK;
    DeviceGuard g(ctx->device);
    cudaStream_t seen[NESF_TRACE_MAX];
    int nseen = 0;
    const int n = t->n < max ? t->n : max;
    for (int i = 0; i < n; i++) {
        NESF_CUDA(cudaEventSynchronize(t->ev[i]));
        float ms = 0.0f;
        NESF_CUDA(cudaEventElapsedTime(&ms, t->ev[0], t->ev[i]));
        int lane = 0;
        while (lane < nseen && seen[lane] != t->stream[i]) lane++;
        if (lane == nseen) seen[nseen++] = t->stream[i];
        std::memset(&out[i], 0, sizeof(out[i]));
        std::snprintf(out[i].name, sizeof(out[i].name), "%s", t->name[i]);
        out[i].stream = lane;
        out[i].t_ms = ms;
    }
    *count = n;
    return NESF_OK;
}

// ------------------------------------------------------------- the autotuner
static int check_tuning(const nesf_tuning& t, const char* who) {
    if (t.solve_block < 0 || t.solve_block > 128 || t.solve_block % 32)
        return fail(NESF_ERR_ARG, "%s: solve_block %d (32, 64, 96 or 128)", who, t.solve_block);
    if (t.deferred_per_sm < 0 || t.deferred_per_sm > 16)
        return fail(NESF_ERR_ARG, "%s: deferred_per_sm %d (1..16)", who, t.deferred_per_sm);
    if (t.infer_per_sm < 0 || t.infer_per_sm > 8)
        return fail(NESF_ERR_ARG, "%s: infer_per_sm %d (1..8)", who, t.infer_per_sm);
    if (t.two_lanes < 0 || t.two_lanes > 1 || t.io_overlap < 0 || t.io_overlap > 1)
        return fail(NESF_ERR_ARG, "%s: two_lanes and io_overlap are 0 or 1", who);
    if (t.pass1_fetch < 0 || t.pass1_fetch > 4)
        return fail(NESF_ERR_ARG, "%s: pass1_fetch %d (1, 2, 3 or 4)", who, t.pass1_fetch);
    if (t.refill_lanes < 0 || t.refill_lanes > 32)
        return fail(NESF_ERR_ARG, "%s: refill_lanes %d (1..32)", who, t.refill_lanes);
    if (t.early_ocean_classify < 0 || t.early_ocean_classify > 3)
        return fail(NESF_ERR_ARG, "%s: early_ocean_classify is 0, 1, 2 or 3", who);
    if (t.ice_deferred_per_sm < 0 || t.ice_deferred_per_sm > 16)
        return fail(NESF_ERR_ARG, "%s: ice_deferred_per_sm %d (0..16)", who, t.ice_deferred_per_sm);
    if (t.cells_per_thread < 0 || t.cells_per_thread > 8)
        return fail(NESF_ERR_ARG, "%s: cells_per_thread %d (1..8)", who, t.cells_per_thread);
    return NESF_OK;
}

// 0 fields take the defaults; the flags are taken as given.
static nesf_tuning complete_tuning(const nesf_tuning& t) {
    nesf_tuning d = default_tuning(), r = t;
    if (!r.solve_block) r.solve_block = d.solve_block;
    if (!r.deferred_per_sm) r.deferred_per_sm = d.deferred_per_sm;
    if (!r.infer_per_sm) r.infer_per_sm = d.infer_per_sm;
    if (!r.pass1_fetch) r.pass1_fetch = d.pass1_fetch;
    if (!r.refill_lanes) r.refill_lanes = d.refill_lanes;
    if (!r.cells_per_thread) r.cells_per_thread = d.cells_per_thread;
    return r;
}

extern "C" int nesf_set_tuning(nesf_context* ctx, const nesf_tuning* t) {
    if (!t) return fail(NESF_ERR_ARG, "nesf_set_tuning: null tuning");
    int r = check_tuning(*t, "nesf_set_tuning");
    if (r || (r = context_or_default(&ctx))) return r;
    std::lock_guard<std::mutex> lk(ctx->lock);
    ctx->tuning = complete_tuning(*t);
    ctx->tuning.step_ms = t->step_ms;
    return NESF_OK;
}

extern "C" int nesf_get_tuning(nesf_context* ctx, nesf_tuning* t) {
    if (!t) return fail(NESF_ERR_ARG, "nesf_get_tuning: null output");
    int r = context_or_default(&ctx);
    if (r) return r;
    std::lock_guard<std::mutex> lk(ctx->lock);
    *t = ctx->tuning;
    return NESF_OK;
}

extern "C" int nesf_autotune(nesf_context* ctx, const nesf_coupling_step_args* a, const nesf_solver_options* opts,
                             int32_t reps, nesf_tuning* out, void* stream) {
    const char* who = "nesf_autotune";
    if (!a) return fail(NESF_ERR_ARG, "%s: null arguments", who);
    if (reps < 1 || reps > 1000) return fail(NESF_ERR_ARG, "%s: reps = %d (1..1000)", who, reps);
    int r = context_or_default(&ctx);
    if (r) return r;
    cudaStream_t s = (cudaStream_t)stream;
    const nesf_tuning start = ctx->tuning;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    {
        DeviceGuard g(ctx->device);
        NESF_CUDA(cudaEventCreate(&e0));
        cudaError_t e = cudaEventCreate(&e1);
        if (e != cudaSuccess) {
            cudaEventDestroy(e0);
            return cuda_fail(e, who);
        }
    }
    // mean step time of a tuning, as the model runs the step: captured as a graph under the
    // tuning, one untimed replay, then `reps` replays (the lanes of a graph schedule
    // differently from the same kernels launched one call at a time)
    auto timed = [&](const nesf_tuning& t, double* ms) -> int {
        ctx->tuning = t;
        nesf_graph* G = nullptr;
        int q = nesf_graph_capture(ctx, a, opts, &G);
        if (q) return q;
        auto done = [&](int rc) { nesf_graph_destroy(G); return rc; };
        if ((q = nesf_graph_launch(G, stream))) return done(q);
        DeviceGuard g(ctx->device);
        cudaError_t e = cudaEventRecord(e0, s);
        for (int i = 0; e == cudaSuccess && i < reps; i++)
            if ((q = nesf_graph_launch(G, stream))) return done(q);
        if (e == cudaSuccess) e = cudaEventRecord(e1, s);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float f = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&f, e0, e1);
        if (e != cudaSuccess) return done(cuda_fail(e, "nesf_autotune"));
        *ms = (double)f / reps;
        return done(NESF_OK);
    };
    const nesf_solver_options o = options_or_default(opts);
    const bool ice = a->ai_params != nullptr;
    const bool warm = o.warm_start && o.mlp && o.precision != NESF_PLAIN_F64;
    const bool fast = o.precision != NESF_PLAIN_F64;
    const bool adaptive = o.precision == NESF_F32_ADAPTIVE;
    nesf_tuning best = complete_tuning(start);
    double best_ms = 0.0;
    r = timed(best, &best_ms);
    // coordinate search: each field's candidates with the others at their best so far; a
    // candidate must beat the best by 1 % (event timings of ~10 ms steps repeat to ~0.5 %)
    struct Axis { int32_t nesf_tuning::*field; std::vector<int32_t> values; bool used; };
    const Axis axes[] = {
        {&nesf_tuning::solve_block, {128, 96, 64, 32}, true},
        {&nesf_tuning::deferred_per_sm, {2, 4, 8, 16}, fast},
        {&nesf_tuning::infer_per_sm, {2, 4, 8}, warm},
        {&nesf_tuning::pass1_fetch, {2, 1, 3, 4}, fast},
        {&nesf_tuning::refill_lanes, {8, 4, 16}, adaptive},
        {&nesf_tuning::two_lanes, {1, 0}, ice},
        {&nesf_tuning::io_overlap, {1, 0}, ice && a->io_params != nullptr},
        {&nesf_tuning::early_ocean_classify, {0, 3, 1, 2}, ice},
        {&nesf_tuning::ice_deferred_per_sm, {0, 1, 2}, ice && fast},
        {&nesf_tuning::cells_per_thread, {1, 2, 4}, adaptive},
    };
    for (const Axis& ax : axes) {
        if (r || !ax.used) continue;
        const int32_t current = best.*(ax.field);
        for (int32_t v : ax.values) {
            if (v == current || r) continue;
            nesf_tuning t = best;
            t.*(ax.field) = v;
            double ms = 0.0;
            if ((r = timed(t, &ms))) break;
            if (ms < 0.99 * best_ms) { best = t; best_ms = ms; }
        }
    }
    {
        DeviceGuard g(ctx->device);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    if (r) {
        ctx->tuning = start;
        return r;
    }
    best.step_ms = best_ms;
    ctx->tuning = best;
    if (out) *out = best;
    return NESF_OK;
}

// ------------------------------------------------------- the tuning cache on disk
// Explicit little-endian serialisation (no struct dumps), so that a file is read the
// same on any host.
namespace {

constexpr char kTuneMagic[8] = {'N', 'E', 'S', 'F', 'T', 'U', 'N', 'E'};
constexpr int kKeyInts = 11;
constexpr uint32_t kKeyBytes = 64 + 4 * kKeyInts;
constexpr int kTuneInts = 10;
constexpr size_t kRecordBytes = kKeyBytes + 4 * kTuneInts + 8;
constexpr size_t kHeaderBytes = 8 + 4 * 4;

void put_u32(std::vector<unsigned char>& b, uint32_t v) {
    for (int i = 0; i < 4; i++) b.push_back((unsigned char)(v >> (8 * i)));
}
void put_u64(std::vector<unsigned char>& b, uint64_t v) {
    for (int i = 0; i < 8; i++) b.push_back((unsigned char)(v >> (8 * i)));
}
uint32_t get_u32(const unsigned char* p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}
uint64_t get_u64(const unsigned char* p) {
    return (uint64_t)get_u32(p) | ((uint64_t)get_u32(p + 4) << 32);
}

void key_ints(const nesf_tuning_key& k, int32_t* v) {
    const int32_t w[kKeyInts] = {k.sm_count, k.compute_capability, k.nx, k.ny, k.hx, k.hy,
                                 k.dtype, k.precision, k.warm_start, k.parts, k.flux_formulation};
    std::memcpy(v, w, sizeof(w));
}
void tune_ints(const nesf_tuning& t, int32_t* v) {
    const int32_t w[kTuneInts] = {t.solve_block, t.deferred_per_sm, t.infer_per_sm, t.two_lanes,
                                  t.io_overlap, t.pass1_fetch, t.refill_lanes, t.early_ocean_classify,
                                  t.ice_deferred_per_sm, t.cells_per_thread};
    std::memcpy(v, w, sizeof(w));
}

void put_key(std::vector<unsigned char>& b, const nesf_tuning_key& k) {
    char name[64];
    std::memset(name, 0, sizeof(name));
    std::memcpy(name, k.device, strnlen(k.device, sizeof(k.device)));
    b.insert(b.end(), name, name + 64);
    int32_t v[kKeyInts];
    key_ints(k, v);
    for (int32_t x : v) put_u32(b, (uint32_t)x);
}

void put_tuning(std::vector<unsigned char>& b, const nesf_tuning& t) {
    int32_t v[kTuneInts];
    tune_ints(t, v);
    for (int32_t x : v) put_u32(b, (uint32_t)x);
    uint64_t bits;
    std::memcpy(&bits, &t.step_ms, 8);
    put_u64(b, bits);
}

nesf_tuning get_tuning_record(const unsigned char* p) {
    int32_t v[kTuneInts];
    for (int i = 0; i < kTuneInts; i++) v[i] = (int32_t)get_u32(p + 4 * i);
    nesf_tuning t;
    std::memset(&t, 0, sizeof(t));
    t.solve_block = v[0]; t.deferred_per_sm = v[1]; t.infer_per_sm = v[2]; t.two_lanes = v[3];
    t.io_overlap = v[4]; t.pass1_fetch = v[5]; t.refill_lanes = v[6]; t.early_ocean_classify = v[7];
    t.ice_deferred_per_sm = v[8]; t.cells_per_thread = v[9];
    const uint64_t bits = get_u64(p + 4 * kTuneInts);
    std::memcpy(&t.step_ms, &bits, 8);
    return t;
}

// The records of a cache file: NESF_OK with `stale` set when the file is missing or
// of another version (no records); an argument error when it is not a cache file.
int read_cache(const char* path, const char* who, std::vector<unsigned char>& records, bool& stale) {
    records.clear();
    stale = false;
    FILE* f = std::fopen(path, "rb");
    if (!f) {
        stale = true;
        return NESF_OK;
    }
    std::vector<unsigned char> all;
    unsigned char buf[4096];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) all.insert(all.end(), buf, buf + n);
    const bool err = std::ferror(f) != 0;
    std::fclose(f);
    if (err) return fail(NESF_ERR_ARG, "%s: cannot read %s", who, path);
    if (all.size() < 8 || std::memcmp(all.data(), kTuneMagic, 8) != 0)
        return fail(NESF_ERR_ARG, "%s: %s is not a tuning cache (no NESFTUNE header)", who, path);
    if (all.size() < kHeaderBytes) return fail(NESF_ERR_ARG, "%s: %s is cut short (header)", who, path);
    const uint32_t version = get_u32(&all[8]), key_bytes = get_u32(&all[12]), fields = get_u32(&all[16]),
                   count = get_u32(&all[20]);
    if (version != NESF_TUNING_VERSION || key_bytes != kKeyBytes || fields != (uint32_t)kTuneInts) {
        stale = true;
        return NESF_OK;
    }
    if (all.size() != kHeaderBytes + (size_t)count * kRecordBytes)
        return fail(NESF_ERR_ARG, "%s: %s holds %zu bytes for %u records (%zu expected)", who, path, all.size(),
                    count, kHeaderBytes + (size_t)count * kRecordBytes);
    records.assign(all.begin() + kHeaderBytes, all.end());
    return NESF_OK;
}

int check_key(const nesf_tuning_key* key, const char* who) {
    if (!key) return fail(NESF_ERR_ARG, "%s: null key", who);
    if (strnlen(key->device, sizeof(key->device)) == sizeof(key->device))
        return fail(NESF_ERR_ARG, "%s: the key's device name is not NUL-terminated", who);
    return NESF_OK;
}

}  // namespace

extern "C" int nesf_tuning_key_of(nesf_context* ctx, const nesf_coupling_step_args* a, const nesf_solver_options* opts,
                                  nesf_tuning_key* key) {
    const char* who = "nesf_tuning_key_of";
    if (!a || !a->ao || !a->ao_params || !key) return fail(NESF_ERR_ARG, "%s: null arguments", who);
    int r = context_or_default(&ctx);
    if (r) return r;
    cudaDeviceProp p;
    NESF_CUDA(cudaGetDeviceProperties(&p, ctx->device));
    const nesf_solver_options o = options_or_default(opts);
    std::memset(key, 0, sizeof(*key));
    std::snprintf(key->device, sizeof(key->device), "%s", p.name);
    key->sm_count = p.multiProcessorCount;
    key->compute_capability = p.major * 10 + p.minor;
    key->nx = a->ao->grid.nx;
    key->ny = a->ao->grid.ny;
    key->hx = a->ao->grid.hx;
    key->hy = a->ao->grid.hy;
    key->dtype = a->ao->dtype;
    key->precision = o.precision;
    key->warm_start = (o.warm_start && o.mlp && o.precision != NESF_PLAIN_F64) ? 1 : 0;
    key->parts = (a->ai_params ? 1 : 0) | (a->io_params ? 2 : 0) | (a->interp ? 4 : 0) |
                 (a->assembly_params ? 8 : 0) | (a->radiation ? 16 : 0);
    key->flux_formulation = a->ao_params->flux_formulation;
    return NESF_OK;
}

extern "C" int nesf_tuning_cache_find(const char* path, const nesf_tuning_key* key, nesf_tuning* out,
                                      int32_t* found) {
    const char* who = "nesf_tuning_cache_find";
    if (!path || !out || !found) return fail(NESF_ERR_ARG, "%s: null arguments", who);
    int r = check_key(key, who);
    if (r) return r;
    *found = 0;
    std::vector<unsigned char> rec;
    bool stale = false;
    if ((r = read_cache(path, who, rec, stale))) return r;
    std::vector<unsigned char> want;
    put_key(want, *key);
    for (size_t off = 0; off + kRecordBytes <= rec.size(); off += kRecordBytes) {
        if (std::memcmp(&rec[off], want.data(), kKeyBytes) != 0) continue;
        *out = get_tuning_record(&rec[off + kKeyBytes]);
        *found = 1;
    }
    return NESF_OK;
}

extern "C" int nesf_tuning_cache_store(const char* path, const nesf_tuning_key* key, const nesf_tuning* tuning) {
    const char* who = "nesf_tuning_cache_store";
    if (!path || !tuning) return fail(NESF_ERR_ARG, "%s: null arguments", who);
    int r = check_key(key, who);
    if (r || (r = check_tuning(*tuning, who))) return r;
    std::vector<unsigned char> rec;
    bool stale = false;
    if ((r = read_cache(path, who, rec, stale))) return r;
    std::vector<unsigned char> want, out;
    put_key(want, *key);
    out.insert(out.end(), kTuneMagic, kTuneMagic + 8);
    put_u32(out, NESF_TUNING_VERSION);
    put_u32(out, kKeyBytes);
    put_u32(out, (uint32_t)kTuneInts);
    put_u32(out, 0);                         // record count, set below
    uint32_t count = 0;
    for (size_t off = 0; off + kRecordBytes <= rec.size(); off += kRecordBytes) {
        if (std::memcmp(&rec[off], want.data(), kKeyBytes) == 0) continue;   // replaced
        out.insert(out.end(), rec.begin() + off, rec.begin() + off + kRecordBytes);
        count++;
    }
    out.insert(out.end(), want.begin(), want.end());
    put_tuning(out, *tuning);
    count++;
    for (int i = 0; i < 4; i++) out[20 + i] = (unsigned char)(count >> (8 * i));
    std::string tmp = std::string(path) + ".tmp";
    FILE* f = std::fopen(tmp.c_str(), "wb");
    if (!f) return fail(NESF_ERR_ARG, "%s: cannot write %s", who, tmp.c_str());
    const bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
    if (std::fclose(f) != 0 || !ok) {
        std::remove(tmp.c_str());
        return fail(NESF_ERR_ARG, "%s: cannot write %s", who, tmp.c_str());
    }
    if (std::rename(tmp.c_str(), path) != 0) {
        std::remove(tmp.c_str());
        return fail(NESF_ERR_ARG, "%s: cannot rename %s over %s", who, tmp.c_str(), path);
    }
    return NESF_OK;
}

extern "C" int nesf_autotune_cached(nesf_context* ctx, const nesf_coupling_step_args* a,
                                    const nesf_solver_options* opts, int32_t reps, const char* path,
                                    nesf_tuning* out, int32_t* from_cache, void* stream) {
    const char* who = "nesf_autotune_cached";
    if (!path || !from_cache) return fail(NESF_ERR_ARG, "%s: null arguments", who);
    int r = context_or_default(&ctx);
    if (r) return r;
    nesf_tuning_key key;
    if ((r = nesf_tuning_key_of(ctx, a, opts, &key))) return r;
    nesf_tuning t;
    int32_t found = 0;
    if ((r = nesf_tuning_cache_find(path, &key, &t, &found))) return r;
    if (found) {
        if ((r = check_tuning(t, who))) return r;
        {
            std::lock_guard<std::mutex> lk(ctx->lock);
            ctx->tuning = complete_tuning(t);
            ctx->tuning.step_ms = t.step_ms;
        }
        if (out) *out = ctx->tuning;
        *from_cache = 1;
        return NESF_OK;
    }
    *from_cache = 0;
    if ((r = nesf_autotune(ctx, a, opts, reps, &t, stream))) return r;
    if (out) *out = t;
    return nesf_tuning_cache_store(path, &key, &t);
}
