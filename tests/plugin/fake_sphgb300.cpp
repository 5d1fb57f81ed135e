// Test infrastructure: a CPU stand-in for libsphgb300 with the entry points that the
// reference-side plugin (splishsplash_gb300/plugin/) calls, implemented over the FP64 oracle
// (oracle/sph_oracle.h).  It lets the plugin's glue -- parameter mapping, upload and download
// of the reference's host vectors, step sizes and time -- run inside the reference's own
// Simulation on a machine without a GPU.  Never shipped, never linked into the product.
#include "sphgb300.h"
#include "sph_oracle.h"

#include <cstring>
#include <string>
#include <vector>

struct sphgb_ctx {
    sphgb_params p{};
    std::vector<double> x, v, a, density, factor, density_adv, kappa, kappa_v, pressure_accel, vdiff, xb, Vb;
    unsigned n = 0, nb = 0;
    double dt = 0.001, time = 0.0;
    sphgb_stats last{};   // statistics of the last step (sphgb_sync)
    std::string err;
};

namespace {
int fail(sphgb_ctx *c, int code, const char *msg)
{
    if (c) c->err = msg;
    return code;
}
template <class T> void copy_in(std::vector<double> &dst, const T *src, size_t m)
{
    dst.resize(m);
    for (size_t i = 0; i < m; i++) dst[i] = static_cast<double>(src[i]);
}
std::vector<double> *field_of(sphgb_ctx *c, int field, int &comps)
{
    comps = 1;
    switch (field) {
    case SPHGB_FIELD_POSITION: comps = 3; return &c->x;
    case SPHGB_FIELD_VELOCITY: comps = 3; return &c->v;
    case SPHGB_FIELD_ACCELERATION: comps = 3; return &c->a;
    case SPHGB_FIELD_DENSITY: return &c->density;
    case SPHGB_FIELD_FACTOR: return &c->factor;
    case SPHGB_FIELD_DENSITY_ADV: return &c->density_adv;
    case SPHGB_FIELD_PRESSURE_RHO2: return &c->kappa;
    case SPHGB_FIELD_PRESSURE_RHO2_V: return &c->kappa_v;
    case SPHGB_FIELD_PRESSURE_ACCEL: comps = 3; return &c->pressure_accel;
    case SPHGB_FIELD_VDIFF: comps = 3; return &c->vdiff;
    default: return nullptr;
    }
}
}  // namespace

extern "C" {

int sphgb_create(const sphgb_config *cfg, sphgb_ctx **out)
{
    if (!cfg || !out || cfg->abi_version != SPHGB_ABI_VERSION || cfg->precision != SPHGB_PRECISION_FP64)
        return SPHGB_ERR_ARGUMENT;
    *out = new sphgb_ctx();
    return SPHGB_OK;
}
int sphgb_destroy(sphgb_ctx *ctx)
{
    delete ctx;
    return SPHGB_OK;
}
const char *sphgb_last_error(const sphgb_ctx *ctx) { return ctx ? ctx->err.c_str() : "no context"; }
int sphgb_default_params(sphgb_params *p)
{
    if (!p) return SPHGB_ERR_ARGUMENT;
    std::memset(p, 0, sizeof(*p));
    return SPHGB_OK;
}
int sphgb_set_params(sphgb_ctx *ctx, const sphgb_params *p)
{
    if (!ctx || !p) return SPHGB_ERR_ARGUMENT;
    ctx->p = *p;
    return SPHGB_OK;
}
int sphgb_upload_boundary(sphgb_ctx *ctx, const double *xb, uint32_t nb)
{
    if (!ctx || (nb && !xb)) return SPHGB_ERR_ARGUMENT;
    copy_in(ctx->xb, xb, 3 * (size_t)nb);
    ctx->nb = nb;
    ctx->Vb.assign(nb, 0.0);
    if (nb && orc_boundary_volume(nb, ctx->xb.data(), 4.0 * ctx->p.particle_radius, 0, ctx->Vb.data()) != 0)
        return fail(ctx, SPHGB_ERR_STATE, "boundary volume");
    return SPHGB_OK;
}
int sphgb_upload_boundary_f32(sphgb_ctx *ctx, const float *, uint32_t)
{
    return fail(ctx, SPHGB_ERR_ARGUMENT, "the stand-in runs the FP64 build only");
}
int sphgb_upload_fluid(sphgb_ctx *ctx, const double *x, const double *v, const uint32_t *id, uint32_t n)
{
    if (!ctx || !x || !v || id) return SPHGB_ERR_ARGUMENT;
    ctx->n = n;
    copy_in(ctx->x, x, 3 * (size_t)n);
    copy_in(ctx->v, v, 3 * (size_t)n);
    for (auto *f : {&ctx->a, &ctx->pressure_accel, &ctx->vdiff}) f->assign(3 * (size_t)n, 0.0);
    for (auto *f : {&ctx->density, &ctx->factor, &ctx->density_adv, &ctx->kappa, &ctx->kappa_v}) f->assign(n, 0.0);
    return SPHGB_OK;
}
int sphgb_upload_fluid_f32(sphgb_ctx *ctx, const float *, const float *, const uint32_t *, uint32_t)
{
    return fail(ctx, SPHGB_ERR_ARGUMENT, "the stand-in runs the FP64 build only");
}
int sphgb_upload_field(sphgb_ctx *ctx, int field, const void *src, int dtype)
{
    int comps = 0;
    std::vector<double> *f = ctx ? field_of(ctx, field, comps) : nullptr;
    if (!f || !src) return SPHGB_ERR_ARGUMENT;
    const size_t m = (size_t)ctx->n * comps;
    if (dtype == SPHGB_DTYPE_F64) copy_in(*f, static_cast<const double *>(src), m);
    else if (dtype == SPHGB_DTYPE_F32) copy_in(*f, static_cast<const float *>(src), m);
    else return SPHGB_ERR_ARGUMENT;
    return SPHGB_OK;
}
int sphgb_download(sphgb_ctx *ctx, int field, void *dst, int dtype)
{
    int comps = 0;
    std::vector<double> *f = ctx ? field_of(ctx, field, comps) : nullptr;
    if (!f || !dst) return SPHGB_ERR_ARGUMENT;
    for (size_t i = 0; i < f->size(); i++) {
        if (dtype == SPHGB_DTYPE_F64) static_cast<double *>(dst)[i] = (*f)[i];
        else if (dtype == SPHGB_DTYPE_F32) static_cast<float *>(dst)[i] = static_cast<float>((*f)[i]);
        else return SPHGB_ERR_ARGUMENT;
    }
    return SPHGB_OK;
}

int sphgb_download_fields(sphgb_ctx *ctx, uint32_t count, const int *fields, void *const *dsts, int dtype)
{
    for (uint32_t k = 0; k < count; k++) {
        const int rc = sphgb_download(ctx, fields[k], dsts[k], dtype);
        if (rc) return rc;
    }
    return SPHGB_OK;
}
int sphgb_set_fluid_phases(sphgb_ctx *ctx, uint32_t nphases, const uint32_t *, const double *)
{
    return nphases <= 1 ? SPHGB_OK : fail(ctx, SPHGB_ERR_ARGUMENT, "one fluid model in the stand-in");
}
int sphgb_num_particles(const sphgb_ctx *ctx, uint32_t *n, uint32_t *nb)
{
    if (!ctx) return SPHGB_ERR_ARGUMENT;
    if (n) *n = ctx->n;
    if (nb) *nb = ctx->nb;
    return SPHGB_OK;
}
int sphgb_set_time_step(sphgb_ctx *ctx, double dt)
{
    if (!ctx || !(dt > 0)) return SPHGB_ERR_ARGUMENT;
    ctx->dt = dt;
    return SPHGB_OK;
}
int sphgb_set_time(sphgb_ctx *ctx, double t)
{
    if (!ctx) return SPHGB_ERR_ARGUMENT;
    ctx->time = t;
    return SPHGB_OK;
}
int sphgb_step(sphgb_ctx *ctx, sphgb_stats *stats)
{
    if (!ctx || !ctx->n) return SPHGB_ERR_STATE;
    const sphgb_params &q = ctx->p;
    orc_params p{};
    p.radius = q.particle_radius;
    p.density0 = q.density0;
    for (int d = 0; d < 3; d++) p.gravity[d] = q.gravity[d];
    p.cfl_method = q.cfl_method;
    p.cfl_factor = q.cfl_factor;
    p.cfl_min = q.cfl_min_time_step;
    p.cfl_max = q.cfl_max_time_step;
    p.min_iterations = q.min_iterations;
    p.max_iterations = q.max_iterations;
    p.max_error = q.max_error;
    p.enable_divergence_solver = q.enable_divergence_solver;
    p.max_iterations_v = q.max_iterations_v;
    p.max_error_v = q.max_error_v;
    p.xsph_fluid = q.xsph;
    p.xsph_boundary = q.xsph_boundary;
    p.viscosity_method = q.viscosity_method;
    p.viscosity = q.viscosity;
    p.viscosity_boundary = q.viscosity_boundary;
    p.visco_max_iter = q.visco_max_iter;
    p.visco_max_error = q.visco_max_error;
    p.fp32_predicate = 0;
    orc_state s{};
    s.n = ctx->n;
    s.nb = ctx->nb;
    s.x = ctx->x.data();
    s.v = ctx->v.data();
    s.a = ctx->a.data();
    s.density = ctx->density.data();
    s.factor = ctx->factor.data();
    s.density_adv = ctx->density_adv.data();
    s.kappa = ctx->kappa.data();
    s.kappa_v = ctx->kappa_v.data();
    s.pressure_accel = ctx->pressure_accel.data();
    s.vdiff = ctx->vdiff.data();
    s.xb = ctx->xb.data();
    s.Vb = ctx->Vb.data();
    s.dt = ctx->dt;
    s.time = ctx->time;
    if (orc_step(&s, &p) != 0) return fail(ctx, SPHGB_ERR_STATE, "oracle step failed");
    ctx->dt = s.dt;
    ctx->time = s.time;
    sphgb_stats &st = ctx->last;
    std::memset(&st, 0, sizeof(st));
    st.iterations = s.iterations;
    st.iterations_v = s.iterations_v;
    st.visco_iterations = s.visco_iterations;
    st.avg_density_err = s.avg_density_err;
    st.avg_density_err_v = s.avg_density_err_v;
    st.visco_error = s.visco_error;
    st.dt_used = s.dt_old;
    st.dt_next = s.dt;
    st.time = s.time;
    if (stats) *stats = st;
    return SPHGB_OK;
}

// the step ran to completion inside sphgb_step: its statistics
int sphgb_sync(sphgb_ctx *ctx, sphgb_stats *stats)
{
    if (!ctx) return SPHGB_ERR_ARGUMENT;
    if (stats) *stats = ctx->last;
    return SPHGB_OK;
}

}  // extern "C"
