/*
 * fdsp_oracle.c -- CPU restatement of libfalcon_dsp's channelizer hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: it is compiled
 * into oracle/_build/libfdsp_oracle.so and loaded by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg, always as the
 * checker and never as the thing measured or shipped.  The product
 * (libfalcon_dsp_gb300) never links or calls it.
 *
 * Every routine restates one reference routine (paths are relative to the
 * reference project root) in plain C99:
 *   - NCO parameters             src/transform/falcon_dsp_freq_shift.cc:194-235
 *   - NCO apply                  src/transform/falcon_dsp_freq_shift.cc:164-192
 *   - resampler initialize       src/transform/falcon_dsp_polyphase_resampler.cc:114-162
 *   - resampler apply            src/transform/falcon_dsp_polyphase_resampler.cc:256-319
 *   - resampler state update     src/transform/falcon_dsp_polyphase_resampler.cc:321-346
 *   - needed_out_count           src/transform/falcon_dsp_polyphase_resampler.cc:216-228
 *   - FIR apply / state          src/transform/falcon_dsp_fir_filter.cc:177-284
 *   - polar discriminator        src/transform/falcon_dsp_polar_discriminator.cc:134-171
 *   - IIR filter                 src/transform/falcon_dsp_iir_filter.cc:67-110, 235-396
 *   - rat_approx                 src/utilities/falcon_dsp_utils.cc:231-294
 *
 * Two arithmetic flavours exist for the NCO and the resampler:
 *   *_f32  mirrors the reference's FP32 data path (FP64 angle, cos/sin in
 *          double rounded to float, complex<float> products and sums);
 *   *_f64  evaluates exactly the same indexing and rollover rule in double
 *          with the FP32 taps promoted to double.  It is the precision oracle
 *          against which SNR in dB is stated.
 *
 * Complex samples are interleaved (re, im) pairs, the layout of
 * std::complex<float> / std::complex<double>.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------------ */
/* NCO frequency shift                                                      */
/* ------------------------------------------------------------------------ */

/* falcon_dsp_freq_shift.cc:194-235: the rollover index is fs/|f| scaled by
 * powers of ten until it reaches 1e5, then rounded; the angular frequency is
 * 2*pi*f/fs in double. */
void orc_freq_shift_params(uint32_t fs, int32_t f, uint32_t *rollover, double *omega)
{
    double r = (double)fs / (double)abs(f);
    while (r < 1e5) {
        r *= 10.0;
    }
    *rollover = (uint32_t)round(r);
    *omega = ((double)f / (double)fs) * 2.0 * M_PI;
}

typedef struct {
    uint32_t rollover;
    double omega;
    uint64_t counter; /* sample counter modulo rollover */
} orc_nco;

orc_nco *orc_nco_new(uint32_t fs, int32_t f)
{
    orc_nco *n = (orc_nco *)calloc(1, sizeof(orc_nco));
    orc_freq_shift_params(fs, f, &n->rollover, &n->omega);
    return n;
}

void orc_nco_free(orc_nco *n) { free(n); }
void orc_nco_reset(orc_nco *n) { n->counter = 0; }
uint32_t orc_nco_rollover(const orc_nco *n) { return n->rollover; }
double orc_nco_omega(const orc_nco *n) { return n->omega; }
uint64_t orc_nco_counter(const orc_nco *n) { return n->counter; }

/* falcon_dsp_freq_shift.cc:164-192 (complex<float> overload). */
void orc_nco_apply_f32(orc_nco *n, const float *in, uint64_t count, float *out)
{
    for (uint64_t i = 0; i < count; ++i) {
        double angle = n->omega * (double)n->counter;
        float c = (float)cos(angle);
        float s = (float)sin(angle);
        float xr = in[2 * i], xi = in[2 * i + 1];
        out[2 * i] = xr * c - xi * s;
        out[2 * i + 1] = xr * s + xi * c;
        n->counter++;
        if (n->counter >= n->rollover) {
            n->counter = 0;
        }
    }
}

/* Same indexing and rollover as orc_nco_apply_f32, evaluated in double. */
void orc_nco_apply_f64(orc_nco *n, const double *in, uint64_t count, double *out)
{
    for (uint64_t i = 0; i < count; ++i) {
        double angle = n->omega * (double)n->counter;
        double c = cos(angle), s = sin(angle);
        double xr = in[2 * i], xi = in[2 * i + 1];
        out[2 * i] = xr * c - xi * s;
        out[2 * i + 1] = xr * s + xi * c;
        n->counter++;
        if (n->counter >= n->rollover) {
            n->counter = 0;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Polyphase resampler                                                      */
/* ------------------------------------------------------------------------ */

typedef struct {
    uint32_t up, down;
    uint32_t padded;   /* tap count rounded up to a multiple of up */
    uint32_t cpp;      /* taps per phase */
    uint32_t phase;    /* coeff_phase, "time" modulo up */
    uint32_t xoffset;  /* carried input offset */
    double *taps;      /* transposed+flipped real parts, padded entries */
    double *state64;   /* cpp-1 complex samples (f64 flavour) */
    float *state32;    /* cpp-1 complex samples (f32 flavour) */
    float *taps32;     /* real parts as float */
} orc_resampler;

/* polyphase_resampler.cc:114-162: pad the taps to a multiple of up, then
 * store phase p flipped at [p*cpp, (p+1)*cpp). */
orc_resampler *orc_resampler_new(uint32_t up, uint32_t down, const float *coeffs, uint32_t ncoeffs)
{
    orc_resampler *r = (orc_resampler *)calloc(1, sizeof(orc_resampler));
    r->up = up;
    r->down = down;
    r->padded = ncoeffs;
    while (r->padded % up) {
        r->padded++;
    }
    r->cpp = r->padded / up;
    r->taps = (double *)calloc(r->padded, sizeof(double));
    r->taps32 = (float *)calloc(r->padded, sizeof(float));
    for (uint32_t ph = 0; ph < up; ++ph) {
        for (uint32_t j = 0; j < r->cpp; ++j) {
            uint32_t src = j * up + ph;
            if (src < ncoeffs) {
                uint32_t dst = (r->cpp - 1 - j) + ph * r->cpp;
                r->taps32[dst] = coeffs[2 * src]; /* real part only is used */
                r->taps[dst] = (double)coeffs[2 * src];
            }
        }
    }
    uint32_t ns = r->cpp > 0 ? r->cpp - 1 : 0;
    r->state64 = (double *)calloc(2 * (size_t)(ns + 1), sizeof(double));
    r->state32 = (float *)calloc(2 * (size_t)(ns + 1), sizeof(float));
    return r;
}

void orc_resampler_free(orc_resampler *r)
{
    if (!r) return;
    free(r->taps);
    free(r->taps32);
    free(r->state64);
    free(r->state32);
    free(r);
}

/* polyphase_resampler.cc:164-172 */
void orc_resampler_reset(orc_resampler *r)
{
    uint32_t ns = r->cpp - 1;
    memset(r->state64, 0, 2 * (size_t)ns * sizeof(double));
    memset(r->state32, 0, 2 * (size_t)ns * sizeof(float));
    r->phase = 0;
    r->xoffset = 0;
}

uint32_t orc_resampler_cpp(const orc_resampler *r) { return r->cpp; }
uint32_t orc_resampler_phase(const orc_resampler *r) { return r->phase; }
uint32_t orc_resampler_xoffset(const orc_resampler *r) { return r->xoffset; }

/* polyphase_resampler.cc:216-228 (kept verbatim in meaning, including its
 * uint32 arithmetic; the apply loop below is what defines the real count). */
uint32_t orc_resampler_needed_out_count(const orc_resampler *r, uint32_t in_count)
{
    uint64_t np = in_count * (uint64_t)r->up;
    uint32_t need = (uint32_t)(np / r->down);
    if ((uint32_t)(r->phase + r->up * r->xoffset) < (np % r->down)) {
        need++;
    }
    return need;
}

/* Count of outputs the apply loop emits for in_count inputs from the
 * current (phase, xoffset), by running the loop's index recurrence. */
uint64_t orc_resampler_loop_out_count(const orc_resampler *r, uint64_t in_count)
{
    int64_t x = r->xoffset;
    uint32_t ph = r->phase;
    uint64_t n = 0;
    while ((uint64_t)x < in_count) {
        n++;
        ph += r->down;
        x += ph / r->up;
        ph %= r->up;
    }
    return n;
}

/* polyphase_resampler.cc:321-346 -- keep the last cpp-1 inputs. */
static void manage_state_f32(orc_resampler *r, const float *in, uint64_t count)
{
    int64_t ns = (int64_t)r->cpp - 1;
    int64_t retain = ns - (int64_t)count;
    if (retain > 0) {
        memmove(r->state32, r->state32 + 2 * (ns - retain), 2 * (size_t)retain * sizeof(float));
        memcpy(r->state32 + 2 * retain, in, 2 * (size_t)count * sizeof(float));
    } else if (ns > 0) {
        memcpy(r->state32, in + 2 * (count - ns), 2 * (size_t)ns * sizeof(float));
    }
}

static void manage_state_f64(orc_resampler *r, const double *in, uint64_t count)
{
    int64_t ns = (int64_t)r->cpp - 1;
    int64_t retain = ns - (int64_t)count;
    if (retain > 0) {
        memmove(r->state64, r->state64 + 2 * (ns - retain), 2 * (size_t)retain * sizeof(double));
        memcpy(r->state64 + 2 * retain, in, 2 * (size_t)count * sizeof(double));
    } else if (ns > 0) {
        memcpy(r->state64, in + 2 * (count - ns), 2 * (size_t)ns * sizeof(double));
    }
}

/* polyphase_resampler.cc:256-319.  Writes at most out_cap outputs and returns
 * how many the loop produced (the caller sizes out with the loop count). */
uint64_t orc_resampler_apply_f32(orc_resampler *r, const float *in, uint64_t count, float *out, uint64_t out_cap)
{
    int64_t x = r->xoffset;
    uint64_t n = 0;
    int64_t cpp = r->cpp;
    int64_t ns = cpp - 1;
    while ((uint64_t)x < count) {
        float ar = 0.0f, ai = 0.0f;
        const float *h = r->taps32 + (size_t)r->phase * cpp;
        int64_t b = x - cpp + 1;
        int64_t off = -b;
        if (off > 0) {
            for (int64_t s = ns - off; s < ns; ++s) {
                ar += r->state32[2 * s] * (*h);
                ai += r->state32[2 * s + 1] * (*h);
                h++;
            }
            b += off;
        }
        for (; b <= x; ++b) {
            ar += in[2 * b] * (*h);
            ai += in[2 * b + 1] * (*h);
            h++;
        }
        if (n < out_cap) {
            out[2 * n] = ar;
            out[2 * n + 1] = ai;
        }
        n++;
        r->phase += r->down;
        x += r->phase / r->up;
        r->phase %= r->up;
    }
    r->xoffset = (uint32_t)(x - (int64_t)count);
    manage_state_f32(r, in, count);
    return n;
}

/* Same recurrence in double (precision oracle). */
uint64_t orc_resampler_apply_f64(orc_resampler *r, const double *in, uint64_t count, double *out, uint64_t out_cap)
{
    int64_t x = r->xoffset;
    uint64_t n = 0;
    int64_t cpp = r->cpp;
    int64_t ns = cpp - 1;
    while ((uint64_t)x < count) {
        double ar = 0.0, ai = 0.0;
        const double *h = r->taps + (size_t)r->phase * cpp;
        int64_t b = x - cpp + 1;
        int64_t off = -b;
        if (off > 0) {
            for (int64_t s = ns - off; s < ns; ++s) {
                ar += r->state64[2 * s] * (*h);
                ai += r->state64[2 * s + 1] * (*h);
                h++;
            }
            b += off;
        }
        for (; b <= x; ++b) {
            ar += in[2 * b] * (*h);
            ai += in[2 * b + 1] * (*h);
            h++;
        }
        if (n < out_cap) {
            out[2 * n] = ar;
            out[2 * n + 1] = ai;
        }
        n++;
        r->phase += r->down;
        x += r->phase / r->up;
        r->phase %= r->up;
    }
    r->xoffset = (uint32_t)(x - (int64_t)count);
    manage_state_f64(r, in, count);
    return n;
}

/* ------------------------------------------------------------------------ */
/* FIR filter with complex taps                                             */
/* ------------------------------------------------------------------------ */

typedef struct {
    uint32_t ntaps;
    float *taps;     /* complex, interleaved */
    float *hist;     /* last ntaps inputs, zero before any input arrived */
} orc_fir;

orc_fir *orc_fir_new(const float *coeffs, uint32_t ntaps)
{
    orc_fir *f = (orc_fir *)calloc(1, sizeof(orc_fir));
    f->ntaps = ntaps;
    f->taps = (float *)malloc(2 * (size_t)ntaps * sizeof(float));
    memcpy(f->taps, coeffs, 2 * (size_t)ntaps * sizeof(float));
    f->hist = (float *)calloc(2 * (size_t)ntaps + 2, sizeof(float));
    return f;
}

void orc_fir_free(orc_fir *f)
{
    if (!f) return;
    free(f->taps);
    free(f->hist);
    free(f);
}

/* fir_filter.cc:136-143 -- the state is emptied, i.e. history reads zero. */
void orc_fir_reset(orc_fir *f) { memset(f->hist, 0, 2 * (size_t)f->ntaps * sizeof(float)); }

/* fir_filter.cc:177-243 and the state update at :245-284.  y[n] =
 * sum_k h[k] x[n-k] with complex products; samples before the first input
 * are zero (the reference's state starts empty).  Returns count. */
uint64_t orc_fir_apply_f32(orc_fir *f, const float *in, uint64_t count, float *out)
{
    uint32_t L = f->ntaps;
    for (uint64_t n = 0; n < count; ++n) {
        float ar = 0.0f, ai = 0.0f;
        for (uint32_t k = 0; k < L; ++k) {
            int64_t idx = (int64_t)n - (int64_t)k;
            float xr, xi;
            if (idx >= 0) {
                xr = in[2 * idx];
                xi = in[2 * idx + 1];
            } else {
                int64_t h = (int64_t)L + idx; /* hist[L-1] is the newest */
                xr = f->hist[2 * h];
                xi = f->hist[2 * h + 1];
            }
            float hr = f->taps[2 * k], hi = f->taps[2 * k + 1];
            ar += xr * hr - xi * hi;
            ai += xr * hi + xi * hr;
        }
        out[2 * n] = ar;
        out[2 * n + 1] = ai;
    }
    /* keep the last L inputs */
    if (count >= L) {
        memcpy(f->hist, in + 2 * (count - L), 2 * (size_t)L * sizeof(float));
    } else if (count > 0) {
        memmove(f->hist, f->hist + 2 * count, 2 * (size_t)(L - count) * sizeof(float));
        memcpy(f->hist + 2 * (L - count), in, 2 * (size_t)count * sizeof(float));
    }
    return count;
}

/* ------------------------------------------------------------------------ */
/* Polar discriminator                                                      */
/* ------------------------------------------------------------------------ */

typedef struct {
    int have_prev;
    float prev_re, prev_im;
} orc_polar;

orc_polar *orc_polar_new(void) { return (orc_polar *)calloc(1, sizeof(orc_polar)); }
void orc_polar_free(orc_polar *p) { free(p); }
void orc_polar_reset(orc_polar *p) { p->have_prev = 0; }

/* polar_discriminator.cc:134-171: out = atan2 of x[n]*conj(x[n-1]); the very
 * first call emits count-1 values.  Returns the number written. */
uint64_t orc_polar_apply_f32(orc_polar *p, const float *in, uint64_t count, float *out)
{
    uint64_t n = 0;
    if (count == 0) return 0;
    if (p->have_prev) {
        float ar = in[0], ai = in[1];
        float br = p->prev_re, bi = -p->prev_im;
        float cr = ar * br - ai * bi, ci = ar * bi + ai * br;
        out[n++] = (float)atan2(ci, cr);
    }
    for (uint64_t i = 1; i < count; ++i) {
        float ar = in[2 * i], ai = in[2 * i + 1];
        float br = in[2 * (i - 1)], bi = -in[2 * (i - 1) + 1];
        float cr = ar * br - ai * bi, ci = ar * bi + ai * br;
        out[n++] = (float)atan2(ci, cr);
    }
    p->have_prev = 1;
    p->prev_re = in[2 * (count - 1)];
    p->prev_im = in[2 * (count - 1) + 1];
    return n;
}

/* ------------------------------------------------------------------------ */
/* IIR filter (direct form, complex<float> taps)                              */
/* ------------------------------------------------------------------------ */

typedef struct {
    uint32_t nb, na;
    float *b, *a;    /* interleaved complex, a[0] = 1 after normalisation */
    float *xs;       /* last nb inputs, oldest first (m_input_state) */
    uint32_t nxs;
    float *ys;       /* last na - 1 outputs, oldest first (m_prev_outputs) */
    uint32_t nys;
} orc_iir;

/* complex<float> product and quotient, one rounding per operation */
static void cmulf(float ar, float ai, float br, float bi, float *cr, float *ci)
{
    float t1 = ar * br, t2 = ai * bi, t3 = ar * bi, t4 = ai * br;
    *cr = t1 - t2;
    *ci = t3 + t4;
}
static void cdivf(float ar, float ai, float br, float bi, float *cr, float *ci)
{
    float d = br * br + bi * bi;
    *cr = (ar * br + ai * bi) / d;
    *ci = (ai * br - ar * bi) / d;
}

/* iir_filter.cc:67-110: b and a divided by a[0] unless a[0].real() == 1. */
orc_iir *orc_iir_new(const float *b, uint32_t nb, const float *a, uint32_t na)
{
    orc_iir *f = (orc_iir *)calloc(1, sizeof(orc_iir));
    if (!f || nb == 0 || na == 0) { free(f); return NULL; }
    f->nb = nb;
    f->na = na;
    f->b = (float *)malloc(2 * (size_t)nb * sizeof(float));
    f->a = (float *)malloc(2 * (size_t)na * sizeof(float));
    f->xs = (float *)calloc(2 * (size_t)nb, sizeof(float));
    f->ys = (float *)calloc(2 * (size_t)na, sizeof(float));
    memcpy(f->b, b, 2 * (size_t)nb * sizeof(float));
    memcpy(f->a, a, 2 * (size_t)na * sizeof(float));
    if (a[0] != 1.0f) {
        for (uint32_t i = 0; i < nb; ++i) cdivf(b[2 * i], b[2 * i + 1], a[0], a[1], &f->b[2 * i], &f->b[2 * i + 1]);
        for (uint32_t i = 1; i < na; ++i) cdivf(a[2 * i], a[2 * i + 1], a[0], a[1], &f->a[2 * i], &f->a[2 * i + 1]);
    }
    return f;
}

void orc_iir_free(orc_iir *f)
{
    if (!f) return;
    free(f->b); free(f->a); free(f->xs); free(f->ys); free(f);
}

void orc_iir_reset(orc_iir *f) { f->nxs = 0; f->nys = 0; }

/* iir_filter.cc:235-396: acc = sum_k b[k] x[n-k] (inputs of this call
 * newest first, then the saved inputs), minus sum_k a[k] y[n-k] over the
 * saved outputs, newest first; one output per input.  Returns count (0 for
 * an empty input, where the reference returns false). */
uint64_t orc_iir_apply_f32(orc_iir *f, const float *in, uint64_t count, float *out)
{
    if (count == 0) return 0;
    for (uint64_t n = 0; n < count; ++n) {
        float accr = 0.f, acci = 0.f, pr, pi;
        uint32_t k = 0;
        if (n < f->nb) {
            for (int64_t i = (int64_t)n; i >= 0; --i, ++k) {
                cmulf(in[2 * i], in[2 * i + 1], f->b[2 * k], f->b[2 * k + 1], &pr, &pi);
                accr = accr + pr; acci = acci + pi;
            }
            for (int64_t s = (int64_t)f->nxs - 1; s >= 0 && k < f->nb; --s, ++k) {
                cmulf(f->xs[2 * s], f->xs[2 * s + 1], f->b[2 * k], f->b[2 * k + 1], &pr, &pi);
                accr = accr + pr; acci = acci + pi;
            }
        } else {
            for (k = 0; k < f->nb; ++k) {
                const uint64_t i = n - k;
                cmulf(in[2 * i], in[2 * i + 1], f->b[2 * k], f->b[2 * k + 1], &pr, &pi);
                accr = accr + pr; acci = acci + pi;
            }
        }
        uint32_t j = 1;
        for (int64_t s = (int64_t)f->nys - 1; s >= 0 && j < f->na; --s, ++j) {
            cmulf(f->ys[2 * s], f->ys[2 * s + 1], f->a[2 * j], f->a[2 * j + 1], &pr, &pi);
            accr = accr - pr; acci = acci - pi;
        }
        out[2 * n] = accr;
        out[2 * n + 1] = acci;
        /* keep the last na - 1 outputs */
        if (f->na > 1) {
            if (f->nys == f->na - 1) {
                memmove(f->ys, f->ys + 2, 2 * (size_t)(f->nys - 1) * sizeof(float));
                f->nys--;
            }
            f->ys[2 * f->nys] = accr;
            f->ys[2 * f->nys + 1] = acci;
            f->nys++;
        }
    }
    /* input state: the last nb inputs (iir_filter.cc:380-396) */
    if (count >= f->nb) {
        memcpy(f->xs, in + 2 * (count - f->nb), 2 * (size_t)f->nb * sizeof(float));
        f->nxs = f->nb;
    } else {
        for (uint64_t i = 0; i < count; ++i) {
            if (f->nxs == f->nb) {
                memmove(f->xs, f->xs + 2, 2 * (size_t)(f->nb - 1) * sizeof(float));
                f->nxs--;
            }
            f->xs[2 * f->nxs] = in[2 * i];
            f->xs[2 * f->nxs + 1] = in[2 * i + 1];
            f->nxs++;
        }
    }
    return count;
}

/* ------------------------------------------------------------------------ */
/* Rational approximation (continued fraction with a denominator cap)        */
/* ------------------------------------------------------------------------ */

/* falcon_dsp_utils.cc:231-294: binary-scale f to an integer ratio d/n, then
 * walk the continued fraction, stopping once the denominator would reach md
 * (taking the half-step convergent when it is at least half the next term). */
void orc_rat_approx(double f, int64_t md, int64_t *num, int64_t *denom)
{
    int64_t h0 = 0, h1 = 1, k0 = 1, k1 = 0;
    int64_t n = 1, d;
    int neg = 0;
    if (md <= 1) {
        *denom = 1;
        *num = (int64_t)f;
        return;
    }
    if (f < 0) {
        neg = 1;
        f = -f;
    }
    while (f != floor(f)) {
        n <<= 1;
        f *= 2;
    }
    d = (int64_t)f;
    for (int i = 0; i < 64; ++i) {
        int64_t a = n ? d / n : 0;
        if (i && !a) break;
        int64_t t = d;
        d = n;
        n = t % n;
        int64_t x = a;
        if (k1 * a + k0 >= md) {
            x = (md - k0) / k1;
            if (x * 2 >= a || k1 >= md) {
                i = 65;
            } else {
                break;
            }
        }
        int64_t h2 = x * h1 + h0;
        h0 = h1;
        h1 = h2;
        int64_t k2 = x * k1 + k0;
        k0 = k1;
        k1 = k2;
    }
    *denom = k1;
    *num = neg ? -h1 : h1;
}
