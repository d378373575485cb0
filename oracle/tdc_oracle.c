/*
 * tdc_oracle.c -- FP64 CPU restatement of the sarlab-tdc focus path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the oracle: it is built and called by
 * tests/, by __graft_entry__.smoke() and by bench.py's cpu_baseline / reference
 * arm, and never by the product library (sarlab-tdc_gb300/), which has no CPU
 * fallback.
 *
 * What it restates (reference paths are relative to the sarlab-tdc project):
 *   - range window           tdc-lib/src/tdckernels.cu:32-50, tuning.h:31
 *   - per-element window     tdc-lib/src/tdckernels.cu:98-131,
 *                            tdc-lib/include/gpumath.h:17-87,
 *                            tdc-lib/include/windowing.h:19-58, tuning.h:38
 *   - reference response     tdc-lib/src/tdckernels.cu:202-216
 *                            ref = w * exp(j*pi*phi), phi = -4 R f / c
 *   - correlate              tdc-lib/src/tdckernels.cu:266-273  raw * conj(ref)
 *   - sum into the pixel     tdc-lib/src/tdckernels.cu:308-314 (NPP sum + addToImage)
 *   - chunk loop + skip test tdc-lib/src/tdcprocessor.cpp:73-156, :347-383
 *                            (PRI_CHUNKSIZE = 128, tuning.h:18), including the
 *                            stale staging rows read for a partial last chunk
 *   - centre wavelength      tdc-lib/src/tdcprocessor.cpp:204-208
 *
 * The reference does all of this in FP32 on the GPU; the oracle does the same
 * arithmetic in FP64 on the values the reference receives (FP32 API inputs are
 * widened exactly), so it is the accuracy yardstick for every GPU kernel.
 *
 * Build: oracle/build.py (gcc -O2 -fopenmp -shared).
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <string.h>
#include <stdlib.h>

#define TDCO_C 299792458.0
#define TDCO_PI 3.14159265358979323846

/* ------------------------------------------------------------------------- */
/* Vector / quaternion helpers (gpumath.h:17-87). Quaternions are (w, x, y, z). */

double tdco_norm3(double x, double y, double z) { return sqrt(x * x + y * y + z * z); }

double tdco_dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

void tdco_q_conj(const double *q, double *out)
{
    out[0] = q[0];
    out[1] = -q[1];
    out[2] = -q[2];
    out[3] = -q[3];
}

/* Hamilton product (gpumath.h:66-72). */
void tdco_q_prod(const double *a, const double *b, double *out)
{
    double r0 = a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
    double r1 = a[0] * b[1] + a[1] * b[0] + a[2] * b[3] - a[3] * b[2];
    double r2 = a[0] * b[2] - a[1] * b[3] + a[2] * b[0] + a[3] * b[1];
    double r3 = a[0] * b[3] + a[1] * b[2] - a[2] * b[1] + a[3] * b[0];
    out[0] = r0;
    out[1] = r1;
    out[2] = r2;
    out[3] = r3;
}

/* v' = q v q*  (gpumath.h:77-87). */
void tdco_q_rot(const double *q, const double *v, double *out)
{
    double vq[4] = {0.0, v[0], v[1], v[2]};
    double qc[4], t[4], r[4];
    tdco_q_conj(q, qc);
    tdco_q_prod(q, vq, t);
    tdco_q_prod(t, qc, r);
    out[0] = r[1];
    out[1] = r[2];
    out[2] = r[3];
}

/* windowing.h:19-24 */
double tdco_doppler_centroid(const double *vel, const double *ant, double lambda)
{
    return 2.0 / lambda * tdco_dot3(vel, ant);
}

/* windowing.h:29-37: 2/lambda * v.(T-P) / |T-P|  (NaN when T == P). */
double tdco_doppler_freq(const double *pos, const double *vel, const double *tgt, double lambda)
{
    double d[3] = {tgt[0] - pos[0], tgt[1] - pos[1], tgt[2] - pos[2]};
    return 2.0 / lambda * tdco_dot3(vel, d) / tdco_norm3(d[0], d[1], d[2]);
}

/* windowing.h:43-58: inclusive |df| <= B/2 test, then Hamming-family taper or 1. */
double tdco_doppler_window(double f_dop, double f_center, double bw, int taper, double a)
{
    double df = f_dop - f_center;
    if (!(fabs(df) <= bw / 2.0)) return 0.0; /* NaN compares false -> 0 */
    if (!taper) return 1.0;
    return a - (1.0 - a) * cos(2.0 * TDCO_PI * df / bw - TDCO_PI);
}

/* tdckernels.cu:32-50: periodic window a - (1-a) cos(2 pi n / N), or all ones. */
void tdco_range_window(double *w, int n_samples, int apply, double a)
{
    for (int n = 0; n < n_samples; ++n) {
        w[n] = apply ? a - (1.0 - a) * cos(2.0 * TDCO_PI * (double)n / (double)n_samples) : 1.0;
    }
}

/*
 * tdcprocessor.cpp:204-208. chirpTime is a float subtraction in the reference
 * (both operands are float), then everything else is double, then cast to float.
 */
float tdco_wavelength_center(const float *sample_times, int n_samples, float mod_rate, float start_freq)
{
    float chirp_time_f = sample_times[n_samples - 1] - sample_times[0];
    double chirp_time = (double)chirp_time_f;
    double end_freq = (double)start_freq + ((double)mod_rate * chirp_time);
    double centre = ((double)start_freq + end_freq) / 2.0;
    return (float)(TDCO_C / centre);
}

/* ------------------------------------------------------------------------- */
/* Problem description. Element (c, s, k) of a trajectory array lives at
 * arr[c * cs + s * ss + k]; ss = 0 describes per-chirp data broadcast over samples.
 * vel == NULL means zero velocity, att == NULL the identity attitude (1,0,0,0). */
typedef struct {
    int n_pri;
    int n_samples;
    const float *raw;          /* [n_pri][n_samples][2] interleaved I/Q */
    const double *sample_times; /* [n_samples] */
    const double *pos;
    long pos_cs, pos_ss;
    const double *vel;
    long vel_cs, vel_ss;
    const double *att;
    long att_cs, att_ss;
    double mod_rate;
    double start_freq;
    double bore[3];
    double lambda;
    const double *grid; /* [n_pix][3] */
    long n_pix;
} tdco_problem;

typedef struct {
    double dop_center;
    double dop_bw;
    int centroid_win;
    int range_win;
    int taper;
    int skip_test; /* apply tdcprocessor.cpp:347-383 per chunk */
    int chunk;     /* PRI_CHUNKSIZE, 128 in the reference */
    double range_a;
    double az_a;
} tdco_opts;

static void traj_get(const double *arr, long cs, long ss, int c, int s, int n, const double *dflt,
                     double *out)
{
    if (!arr) {
        for (int k = 0; k < n; ++k) out[k] = dflt[k];
        return;
    }
    const double *p = arr + (long)c * cs + (long)s * ss;
    for (int k = 0; k < n; ++k) out[k] = p[k];
}

static const double ZERO3[3] = {0.0, 0.0, 0.0};
static const double QIDENT[4] = {1.0, 0.0, 0.0, 0.0};

static double centre_of(const tdco_problem *p, const tdco_opts *o, const double *vel, const double *att)
{
    if (!o->centroid_win) return o->dop_center;
    double ant[3];
    tdco_q_rot(att, p->bore, ant);
    return tdco_doppler_centroid(vel, ant, p->lambda);
}

/*
 * Index of the PRI whose trajectory the reference's skip test reads for chunk
 * `chunk_idx`, chunk-relative row `row`: rows past the valid PRIs of a partial
 * chunk still hold the previous chunk's data (stageNextChunk copies only the
 * valid rows, tdcprocessor.cpp:320-345). Returns -1 for a row that was never
 * written (single partial chunk): its contents are taken as zeros.
 */
int tdco_skip_row_pri(int n_pri, int chunk, int chunk_idx, int row)
{
    long base = (long)chunk_idx * chunk;
    long valid = n_pri - base;
    if (valid > chunk) valid = chunk;
    if (row < valid) return (int)(base + row);
    if (chunk_idx == 0) return -1;
    return (int)(base - chunk + row);
}

/* tdcprocessor.cpp:355-362: the 3 x 3 (PRI, sample) points of the skip test. */
void tdco_skip_points(int n_samples, int chunk, int *rows, int *samples)
{
    int pri_step = chunk / 2;
    int sample_step = n_samples / 2;
    for (int i = 0; i < 3; ++i) {
        int r = i * pri_step - 1;
        rows[i] = r < 0 ? 0 : r;
        int s = i * sample_step - 1;
        samples[i] = s < 0 ? 0 : s;
    }
}

/*
 * tdcprocessor.cpp:347-383. Returns 1 when the chunk is processed for this
 * target. std::min_element keeps element 0 when it is NaN (NaN never compares
 * less), and never selects a later NaN; the final `<= B/2` is false for NaN.
 */
int tdco_window_is_nonzero(const tdco_problem *p, const tdco_opts *o, int chunk_idx, const double *tgt)
{
    int rows[3], samples[3];
    tdco_skip_points(p->n_samples, o->chunk, rows, samples);
    double vals[9];
    for (int i = 0; i < 3; ++i) {
        int pri = tdco_skip_row_pri(p->n_pri, o->chunk, chunk_idx, rows[i]);
        for (int j = 0; j < 3; ++j) {
            double pos[3], vel[3], att[4];
            if (pri < 0) {
                memset(pos, 0, sizeof pos);
                memset(vel, 0, sizeof vel);
                memset(att, 0, sizeof att);
            } else {
                traj_get(p->pos, p->pos_cs, p->pos_ss, pri, samples[j], 3, ZERO3, pos);
                traj_get(p->vel, p->vel_cs, p->vel_ss, pri, samples[j], 3, ZERO3, vel);
                traj_get(p->att, p->att_cs, p->att_ss, pri, samples[j], 4, QIDENT, att);
            }
            double fc = centre_of(p, o, vel, att);
            vals[i * 3 + j] = fabs(tdco_doppler_freq(pos, vel, tgt, p->lambda) - fc);
        }
    }
    double m = vals[0];
    for (int k = 1; k < 9; ++k) {
        if (vals[k] < m) m = vals[k];
    }
    return m <= o->dop_bw / 2.0;
}

/* Per-chirp / per-sample window pieces (tdckernels.cu:104-131). */
static double element_waz(const tdco_problem *p, const tdco_opts *o, int c, int s, const double *tgt)
{
    double pos[3], vel[3], att[4];
    traj_get(p->pos, p->pos_cs, p->pos_ss, c, s, 3, ZERO3, pos);
    traj_get(p->vel, p->vel_cs, p->vel_ss, c, s, 3, ZERO3, vel);
    traj_get(p->att, p->att_cs, p->att_ss, c, s, 4, QIDENT, att);
    double fc = centre_of(p, o, vel, att);
    double fd = tdco_doppler_freq(pos, vel, tgt, p->lambda);
    return tdco_doppler_window(fd, fc, o->dop_bw, o->taper, o->az_a);
}

/* Round-trip phase in cycles, reduced to [-0.5, 0.5]: 2 R f / c. */
static double phase_cycles(double r, double f)
{
    double cyc = 2.0 * r * f / TDCO_C;
    return cyc - nearbyint(cyc);
}

/*
 * Focus pixels pix_idx[0..n_out) (all pixels 0..n_out when pix_idx is NULL):
 *   I(T) = sum over processed chunks, chirps c, samples s of
 *          w_r[s] * w_az(c, s, T) * raw[c, s] * exp(+j 2 pi * 2 R_cs(T) f_s / c0),
 *   f_s = start_freq + mod_rate * t_s,
 * i.e. raw * conj(ref) with ref = w * exp(j pi phi), phi = -4 R f / c0.
 * out receives interleaved (Re, Im) doubles.
 */
int tdco_focus(const tdco_problem *p, const tdco_opts *o, const long *pix_idx, long n_out, double *out,
               int n_threads)
{
    if (!p || !o || !out || p->n_pri <= 0 || p->n_samples <= 0 || o->chunk <= 0) return -1;
    const int S = p->n_samples, C = p->n_pri;
    double *wr = (double *)malloc(sizeof(double) * S);
    double *fs = (double *)malloc(sizeof(double) * S);
    if (!wr || !fs) {
        free(wr);
        free(fs);
        return -2;
    }
    tdco_range_window(wr, S, o->range_win, o->range_a);
    for (int s = 0; s < S; ++s) fs[s] = p->start_freq + p->mod_rate * p->sample_times[s];
    const int n_chunks = (C + o->chunk - 1) / o->chunk;
    const int chirp_const_pos = (p->pos_ss == 0);
    const int chirp_const_win = chirp_const_pos && (!p->vel || p->vel_ss == 0) && (!p->att || p->att_ss == 0);
    if (n_threads <= 0) n_threads = 1;

#pragma omp parallel for schedule(dynamic, 1) num_threads(n_threads)
    for (long i = 0; i < n_out; ++i) {
        long pix = pix_idx ? pix_idx[i] : i;
        const double *tgt = p->grid + 3 * pix;
        double acc_re = 0.0, acc_im = 0.0;
        for (int k = 0; k < n_chunks; ++k) {
            if (o->skip_test && !tdco_window_is_nonzero(p, o, k, tgt)) continue;
            int c_end = (k + 1) * o->chunk;
            if (c_end > C) c_end = C;
            for (int c = k * o->chunk; c < c_end; ++c) {
                const float *row = p->raw + 2L * S * c;
                double waz_c = chirp_const_win ? element_waz(p, o, c, 0, tgt) : 0.0;
                double r_c = 0.0;
                if (chirp_const_pos) {
                    const double *pc = p->pos + (long)c * p->pos_cs;
                    r_c = tdco_norm3(pc[0] - tgt[0], pc[1] - tgt[1], pc[2] - tgt[2]);
                }
                if (chirp_const_win && waz_c == 0.0) continue;
                for (int s = 0; s < S; ++s) {
                    double w = wr[s] * (chirp_const_win ? waz_c : element_waz(p, o, c, s, tgt));
                    if (w == 0.0) continue;
                    double r = r_c;
                    if (!chirp_const_pos) {
                        const double *ps = p->pos + (long)c * p->pos_cs + (long)s * p->pos_ss;
                        r = tdco_norm3(ps[0] - tgt[0], ps[1] - tgt[1], ps[2] - tgt[2]);
                    }
                    double th = 2.0 * TDCO_PI * phase_cycles(r, fs[s]);
                    double cs = cos(th), sn = sin(th);
                    double xr = w * (double)row[2 * s], xi = w * (double)row[2 * s + 1];
                    acc_re += xr * cs - xi * sn;
                    acc_im += xr * sn + xi * cs;
                }
            }
        }
        out[2 * i] = acc_re;
        out[2 * i + 1] = acc_im;
    }
    free(wr);
    free(fs);
    return 0;
}

/*
 * Gradient of a real loss L(I) with respect to per-chirp antenna offsets d_c
 * (positions P_c + d_c; requires per-chirp positions, pos_ss == 0). g holds
 * dL/dRe I + j dL/dIm I per output pixel (interleaved), as torch stores the
 * gradient of a complex tensor. The Doppler window and skip test are held fixed
 * (they are evaluated at the offset positions but not differentiated):
 *   dL/dd_c = sum_T Re(conj(g_T) * w_c(T) * j 2 pi * D_c(T)) * u_c(T),
 *   D_c(T) = sum_s (2 f_s / c0) w_r[s] raw[c, s] exp(j theta_cs),  u = (P_c + d_c - T) / R.
 * No reference counterpart (the reference has no gradient path).
 */
int tdco_adjoint_offsets(const tdco_problem *p, const tdco_opts *o, const double *offsets, const long *pix_idx,
                         long n_out, const double *g, double *grad, int n_threads)
{
    if (!p || !o || !g || !grad || p->pos_ss != 0 || p->n_pri <= 0 || p->n_samples <= 0) return -1;
    const int S = p->n_samples, C = p->n_pri;
    double *wr = (double *)malloc(sizeof(double) * S);
    double *fs = (double *)malloc(sizeof(double) * S);
    if (!wr || !fs) {
        free(wr);
        free(fs);
        return -2;
    }
    tdco_range_window(wr, S, o->range_win, o->range_a);
    for (int s = 0; s < S; ++s) fs[s] = p->start_freq + p->mod_rate * p->sample_times[s];
    const int chirp_const_win = (!p->vel || p->vel_ss == 0) && (!p->att || p->att_ss == 0);
    if (!chirp_const_win) {
        free(wr);
        free(fs);
        return -3;
    }
    if (n_threads <= 0) n_threads = 1;

    /* The shifted trajectory the forward pass sees. */
    double *shifted = (double *)malloc(sizeof(double) * 3 * C);
    if (!shifted) {
        free(wr);
        free(fs);
        return -2;
    }
    for (int c = 0; c < C; ++c)
        for (int k = 0; k < 3; ++k)
            shifted[3 * c + k] = p->pos[(long)c * p->pos_cs + k] + (offsets ? offsets[3 * c + k] : 0.0);
    tdco_problem q = *p;
    q.pos = shifted;
    q.pos_cs = 3;
    q.pos_ss = 0;

#pragma omp parallel for schedule(dynamic, 1) num_threads(n_threads)
    for (int c = 0; c < C; ++c) {
        const float *row = q.raw + 2L * S * c;
        const double *pc = shifted + 3 * c;
        int chunk_idx = c / o->chunk;
        double gx = 0.0, gy = 0.0, gz = 0.0;
        for (long i = 0; i < n_out; ++i) {
            long pix = pix_idx ? pix_idx[i] : i;
            const double *tgt = q.grid + 3 * pix;
            if (o->skip_test && !tdco_window_is_nonzero(&q, o, chunk_idx, tgt)) continue;
            double waz = element_waz(&q, o, c, 0, tgt);
            if (waz == 0.0) continue;
            double d[3] = {pc[0] - tgt[0], pc[1] - tgt[1], pc[2] - tgt[2]};
            double r = tdco_norm3(d[0], d[1], d[2]);
            if (r == 0.0) continue;
            double dre = 0.0, dim = 0.0;
            for (int s = 0; s < S; ++s) {
                double th = 2.0 * TDCO_PI * phase_cycles(r, fs[s]);
                double cs = cos(th), sn = sin(th);
                double gs = 2.0 * fs[s] / TDCO_C;
                double xr = wr[s] * (double)row[2 * s], xi = wr[s] * (double)row[2 * s + 1];
                dre += gs * (xr * cs - xi * sn);
                dim += gs * (xr * sn + xi * cs);
            }
            /* dI/dR = waz * j 2 pi D ; Re(conj(g) * j 2 pi waz D) */
            double jr = -2.0 * TDCO_PI * waz * dim, ji = 2.0 * TDCO_PI * waz * dre;
            double gre = g[2 * i], gim = g[2 * i + 1];
            double dl_dr = gre * jr + gim * ji;
            gx += dl_dr * d[0] / r;
            gy += dl_dr * d[1] / r;
            gz += dl_dr * d[2] / r;
        }
        grad[3 * c] = gx;
        grad[3 * c + 1] = gy;
        grad[3 * c + 2] = gz;
    }
    free(shifted);
    free(wr);
    free(fs);
    return 0;
}
