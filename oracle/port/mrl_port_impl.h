/*
 * mrl_port_impl.h -- body of the CPU oracle, included by mrl_port.c once per
 * precision with REAL = float or double and PORT_FN set to the exported
 * name.  TEST INFRASTRUCTURE: see mrl_port.h.
 */


typedef struct {
    REAL dt;
    REAL amp[MRL_PORT_MAX_TX], phase[MRL_PORT_MAX_TX], freq[MRL_PORT_MAX_TX];
    REAL gz, gy, gx;
    int adc;
} PORT_T(step);

/* Closed-form rotation of one free isochromat for one step.  RF on:
 * rotation by alpha about the effective field tilted by beta from the
 * transverse plane at azimuth -phi (BlochKernel.cuh:194-255, the CPU kernel
 * BlochKernel.h:57-310 evaluates the same closed form with IPP vector ops).
 * RF off: precession by dW*dt (BlochKernel.cuh:258-264). */
static void PORT_T(rotate)(REAL *mx, REAL *my, REAL *mz, REAL dW, const PORT_T(step) *st,
                            int tx_num, REAL gyro, const REAL *mg, const REAL *pe, REAL rf_sum) {
    REAL Mx = *mx, My = *my, Mz = *mz;
    if (rf_sum != 0) {
        REAL b1, ph;
        if (tx_num == 1) {
            dW += (REAL)(2 * PI * (double)st->freq[0]);
            b1 = mg[0] * st->amp[0];
            ph = pe[0] + st->phase[0];
        } else {
            REAL re = 0, im = 0;
            for (int c = 0; c < tx_num; ++c) {
                if (st->amp[c] != 0) {
                    dW += (REAL)(2 * PI * (double)st->freq[c]);
                    REAL a = mg[c] * st->amp[c];
                    REAL p = pe[c] + st->phase[c];
                    re += a * RCOS(p);
                    im += a * RSIN(p);
                }
            }
            b1 = RSQRT((REAL)(re * re + im * im));
            ph = RATAN2(im, re);
        }
        REAL g1 = b1 * gyro;
        REAL alpha = RSQRT((REAL)(dW * dW + g1 * g1)) * st->dt;
        REAL beta = RATAN((REAL)(dW / g1));
        REAL sa = RSIN(alpha), ca = RCOS(alpha);
        REAL sb = RSIN(beta), cb = RCOS(beta);
        REAL cp = RCOS(-ph), sp = RSIN(-ph);
        REAL b1x = cb * cb * cp - sb * (sa * sp - ca * cp * sb);
        REAL b2x = sp * cb * cb + sb * (cp * sa + ca * sb * sp);
        REAL nx = Mx * (cp * b1x + sp * (ca * sp + cp * sa * sb)) - My * (sp * b1x - cp * (ca * sp + cp * sa * sb)) +
                  Mz * (cb * (sa * sp - ca * cp * sb) + cb * cp * sb);
        REAL ny = My * (sp * b2x + cp * (ca * cp - sa * sb * sp)) - Mx * (cp * b2x - sp * (ca * cp - sa * sb * sp)) +
                  Mz * (cb * (cp * sa + ca * sb * sp) - cb * sb * sp);
        REAL nz = Mx * (cp * (cb * sb - ca * cb * sb) - cb * sa * sp) - My * (sp * (cb * sb - ca * cb * sb) + cb * cp * sa) +
                  Mz * (ca * cb * cb + sb * sb);
        *mx = nx;
        *my = ny;
        *mz = nz;
    } else {
        REAL a = dW * st->dt;
        REAL s = RSIN(a), c = RCOS(a);
        *mx = Mx * c + My * s;
        *my = My * c - Mx * s;
        *mz = Mz;
    }
}

/* Single-pool RF rotation in the CPU engine's exact operation order
 * (BlochKernel.h:57-310): the same closed form as rotate() but evaluated as
 * the reference's sequence of IPP vector ops, so that a single-precision
 * build rounds the way the reference engine does. */
static void PORT_T(rotate_cpu)(REAL *mx, REAL *my, REAL *mz, REAL dW, const PORT_T(step) *st, int tx_num,
                                REAL gyro, const REAL *mg, const REAL *pe) {
    REAL b1, b2;
    if (tx_num == 1) {
        b1 = mg[0] * st->amp[0];
        b2 = pe[0] + st->phase[0];
        dW += (REAL)((double)(st->freq[0] * 2) * PI);
        b1 = b1 * gyro;
        b2 = b2 * (REAL)-1;
    } else {
        REAL b5 = 0, b6 = 0;
        for (int c = 0; c < tx_num; ++c) {
            if (st->amp[c] != 0) {
                REAL a1 = mg[c] * st->amp[c];
                REAL a2 = pe[c] + st->phase[c];
                b5 += a1 * RCOS(a2);
                b6 += a1 * RSIN(a2);
                dW += (REAL)((double)(st->freq[c] * 2) * PI);
            }
        }
        b1 = RSQRT(b5 * b5 + b6 * b6);
        b2 = RATAN2(b6, b5);
        b1 = b1 * gyro;
        b2 = b2 * (REAL)-1;
    }
    REAL beta = RATAN(dW / b1);
    REAL q = dW * dW;
    b1 = b1 * b1;
    q = q + b1;
    q = RSQRT(q);
    REAL alpha = q * st->dt;
    const REAL SA = RSIN(alpha), SB = RSIN(beta), CA = RCOS(alpha), CB = RCOS(beta);
    const REAL SP = RSIN(b2), mSP = SP * (REAL)-1, CP = RCOS(b2), mCP = CP * (REAL)-1;
    const REAL Mx = *mx, My = *my, Mz = *mz;
    REAL x1, x2, x3, x4, buf;
    /* Mx */
    x1 = SB * CA; x1 = x1 * mCP; x3 = SA * SP; x1 = x1 + x3; x1 = x1 * SB; x1 = x1 * (REAL)-1;
    x3 = CB * CB; x3 = x3 * CP; x1 = x1 + x3; x3 = x1;
    x1 = x1 * CP; x3 = x3 * SP;
    x2 = SA * SB; x2 = x2 * CP; x4 = CA * SP; x2 = x2 + x4; x4 = x2;
    x2 = x2 * SP; x4 = x4 * mCP;
    x2 = x2 + x1; x2 = x2 * Mx;
    x4 = x4 + x3; x4 = x4 * My; x4 = x4 * (REAL)-1;
    buf = x2 + x4;
    x1 = SB * CB; x1 = x1 * CP;
    x2 = SB * CA; x2 = x2 * mCP;
    x3 = SA * SP;
    x2 = x2 + x3; x2 = x2 * CB;
    x1 = x1 + x2; x1 = x1 * Mz;
    const REAL nx = buf + x1;
    /* My */
    x1 = CA * SB; x1 = x1 * SP; x3 = SA * CP; x1 = x1 + x3; x1 = x1 * SB;
    x3 = CB * CB; x3 = x3 * SP; x1 = x1 + x3; x3 = x1;
    x1 = x1 * SP; x3 = x3 * CP;
    x2 = SA * SB; x2 = x2 * mSP; x4 = CA * CP; x2 = x2 + x4; x4 = x2;
    x2 = x2 * CP; x4 = x4 * mSP;
    x2 = x2 + x1; x2 = x2 * My;
    x4 = x4 + x3; x4 = x4 * Mx; x4 = x4 * (REAL)-1;
    buf = x2 + x4;
    x1 = CB * SB; x1 = x1 * mSP;
    x2 = CA * SB; x2 = x2 * SP;
    x3 = SA * CP;
    x2 = x2 + x3; x2 = x2 * CB;
    x1 = x1 + x2; x1 = x1 * Mz;
    const REAL ny = buf + x1;
    /* Mz */
    x1 = CA * CB; x1 = x1 * SB; x1 = x1 * (REAL)-1;
    x3 = CB * SB; x1 = x1 + x3; x3 = x1;
    x1 = x1 * CP; x3 = x3 * SP;
    x2 = CB * SA; x2 = x2 * mSP;
    x4 = CB * SA; x4 = x4 * CP;
    x2 = x2 + x1; x2 = x2 * Mx;
    x4 = x4 + x3; x4 = x4 * My; x4 = x4 * (REAL)-1;
    buf = x2 + x4;
    x1 = SB * SB;
    x2 = CB * CB; x2 = x2 * CA;
    x1 = x1 + x2; x1 = x1 * Mz;
    const REAL nz = buf + x1;
    *mx = nx;
    *my = ny;
    *mz = nz;
}

/* Super-Lorentzian absorption lineshape of a bound pool, by the reference's
 * 1000-point rectangle rule over u in [0, 1) (BlochKernelMT.cuh:348-358;
 * u advances by 0.001 in single precision there, and here for REAL=float). */
static REAL PORT_T(lineshape)(REAL rf_freq, REAL db0, REAL gyro, REAL t2b) {
    REAL u = 0, g = 0;
    for (int p = 0; p < 1000; ++p) {
        REAL den = (REAL)(3 * (double)u * (double)u - 1);
        REAL x = (REAL)(((2 * PI * (double)rf_freq + (double)(db0 * gyro)) * (double)t2b) / (double)den);
        g = (REAL)((double)g + sqrt(2 / PI) * (double)(t2b / (REAL)fabs((double)den)) *
                                   (double)REXP((REAL)(-2 * x * x)) * 0.001);
        u = (REAL)((double)u + 0.001);
    }
    return g;
}

/* Saturation rate W of a bound pool (BlochKernelMT.cuh:336-399). */
static REAL PORT_T(bound_w)(const PORT_T(step) *st, int tx_num, REAL gyro, const REAL *mg, REAL db0, REAL t2b) {
    if (tx_num == 1) {
        REAL b1 = mg[0] * (REAL)fabs((double)st->amp[0]);
        REAL g = PORT_T(lineshape)(st->freq[0], db0, gyro, t2b);
        return (REAL)(PI * (double)((b1 * gyro) * (b1 * gyro)) * (double)g);
    }
    REAL w = 0, n = 0;
    for (int c = 0; c < tx_num; ++c) {
        if (st->amp[c] != 0) {
            REAL b1 = mg[c] * (REAL)fabs((double)st->amp[c]);
            REAL g = PORT_T(lineshape)(st->freq[c], db0, gyro, t2b);
            w += (REAL)(PI * (double)((b1 * gyro) * (b1 * gyro)) * (double)g);
            n += 1;
        }
    }
    return w / n;
}

static REAL PORT_T(relax_exp)(REAL dt, REAL t) {
    /* exp(-dt/T) with the CPU kernel's clamp of the exponent at -200
     * (BlochKernel.h:348-358) */
    REAL e = -(dt * ((REAL)1 / t));
    if (e < (REAL)-200) e = (REAL)-200;
    return REXP((REAL)e);
}

/* Exchange rate from pool t to pool p of voxel v in each model's K layout:
 * ME channel t*P+p, GM channel p*P+t (BlochKernelME.cuh, BlochKernelGM.cuh);
 * MT channel 1 = K12 (0 -> 1), 2 = K21 (1 -> 0) (BlochKernelMT.cuh:324-407);
 * CEST channel 0 = 0 -> MT, P-1 = MT -> 0, t-1 = 0 -> t, t+P-2 = t -> 0
 * (BlochKernelCEST.cuh:364-600). */
static double PORT_T(rate)(const mrl_port_args *a, long V, int v, int t, int p) {
    const int P = a->type_num;
    long ch = -1;
    switch (a->model) {
    case MRL_PORT_ME: ch = (long)t * P + p; break;
    case MRL_PORT_GM: ch = (long)p * P + t; break;
    case MRL_PORT_MT: ch = (t == 0 && p == 1) ? 1 : (t == 1 && p == 0) ? 2 : -1; break;
    case MRL_PORT_CEST:
        if (t == 0) ch = p == 1 ? 0 : p - 1;
        else if (p == 0) ch = t == 1 ? P - 1 : t + P - 2;
        break;
    default: break;
    }
    return ch < 0 ? 0.0 : (double)a->k[ch * V + v];
}

/* One dt > 0 step of one isochromat group (voxel v, spin s) for the model. */
static void PORT_T(update)(const mrl_port_args *a, REAL *MX, REAL *MY, REAL *MZ, long V, int v, int s,
                           const PORT_T(step) *st, REAL rf_sum, REAL gyro) {
    const int P = a->type_num, S = a->spin_num, tx = a->tx_num;
    REAL mg[MRL_PORT_MAX_TX], pe[MRL_PORT_MAX_TX];
    for (int c = 0; c < tx; ++c) {
        mg[c] = a->tx_mg[(long)c * V + v];
        pe[c] = a->tx_pe[(long)c * V + v];
    }
    const REAL db0 = a->db0[v];
    const REAL gterm_z = a->gzgrid[v], gterm_y = a->gygrid[v], gterm_x = a->gxgrid[v];
    const REAL dt = st->dt;
#define IDX(t) ((long)(t) * S * V + (long)s * V + v)
#define PIDX(t) ((long)(t) * V + v)
#define DW(t)                                                                                    \
    ((REAL)(db0 * gyro + (REAL)a->dwrnd[IDX(t)] + (REAL)(2 * PI * (double)(REAL)a->cs[t]) +         \
            gterm_z * (st->gz * gyro) + gterm_y * (st->gy * gyro) + gterm_x * (st->gx * gyro)))

    if (a->model == MRL_PORT_NORMAL) {
        for (int t = 0; t < P; ++t) {
            REAL T1 = a->t1[PIDX(t)], T2 = a->t2[PIDX(t)], rho = a->rho[PIDX(t)];
            if (T2 == 0 || T1 == 0 || rho == 0) continue;
            long i = IDX(t);
            REAL x = MX[i], y = MY[i], z = MZ[i];
            if (rf_sum != 0)
                PORT_T(rotate_cpu)(&x, &y, &z, DW(t), st, tx, gyro, mg, pe);
            else
                PORT_T(rotate)(&x, &y, &z, DW(t), st, tx, gyro, mg, pe, rf_sum);
            REAL e2 = PORT_T(relax_exp)(dt, T2), e1 = PORT_T(relax_exp)(dt, T1);
            MX[i] = x * e2;
            MY[i] = y * e2;
            MZ[i] = z * e1 + ((REAL)1 - e1) * (rho / (REAL)S);
        }
        return;
    }

    const int mtc = a->model == MRL_PORT_MT || a->model == MRL_PORT_CEST;
    if ((a->model == MRL_PORT_ME || a->model == MRL_PORT_GM || mtc) && a->exact) {
        /* exact relaxation-exchange propagator after the rotation of every
         * free pool and the saturation of every bound (GM TypeFlag 1; MT /
         * CEST pool 1) pool; a bound pool has no transverse generator (its
         * transverse magnetisation is held, and no free pool takes
         * transverse inflow from it) but takes part in the longitudinal one.
         * MT / CEST keep their models' transverse map: a free pool's
         * transverse magnetisation does not flow out to the bound pool
         * (BlochKernelMT.cuh:324-333, BlochKernelCEST.cuh:364-395); only
         * voxels whose pool 0 is active evolve */
        if (mtc && (a->t2[PIDX(0)] == 0 || a->t1[PIDX(0)] == 0 || a->rho[PIDX(0)] == 0)) return;
        REAL rx[MRL_PORT_MAX_POOL], ry[MRL_PORT_MAX_POOL], rz[MRL_PORT_MAX_POOL];
        double At[MRL_PORT_MAX_POOL * MRL_PORT_MAX_POOL] = {0}, Al[MRL_PORT_MAX_POOL * MRL_PORT_MAX_POOL] = {0};
        double Ft[MRL_PORT_MAX_POOL * MRL_PORT_MAX_POOL], Fl[MRL_PORT_MAX_POOL * MRL_PORT_MAX_POOL];
        double Xt[MRL_PORT_MAX_POOL * MRL_PORT_MAX_POOL], Xl[MRL_PORT_MAX_POOL * MRL_PORT_MAX_POOL];
        double b[MRL_PORT_MAX_POOL] = {0};
        int on[MRL_PORT_MAX_POOL], bnd[MRL_PORT_MAX_POOL];
        for (int t = 0; t < P; ++t)
            bnd[t] = (a->model == MRL_PORT_GM && (int)a->type_flag[t] == 1) || (mtc && t == 1);
        for (int t = 0; t < P; ++t) {
            REAL T1 = a->t1[PIDX(t)], T2 = a->t2[PIDX(t)], rho = a->rho[PIDX(t)];
            on[t] = !(T2 == 0 || T1 == 0 || rho == 0);
            rx[t] = MX[IDX(t)];
            ry[t] = MY[IDX(t)];
            rz[t] = MZ[IDX(t)];
            if (!on[t]) continue;
            if (!bnd[t]) {
                PORT_T(rotate)(&rx[t], &ry[t], &rz[t], DW(t), st, tx, gyro, mg, pe, rf_sum);
                At[t * P + t] = -1.0 / (double)T2;
            } else if (rf_sum != 0) {
                REAL w = PORT_T(bound_w)(st, tx, gyro, mg, db0, T2);
                rz[t] = rz[t] * REXP((REAL)(-w * dt));
            }
            Al[t * P + t] = -1.0 / (double)T1;
            b[t] = (double)rho / ((double)S * (double)T1);
            for (int p = 0; p < P; ++p) {
                if (p == t) continue; /* a self rate moves nothing */
                const double kgo = PORT_T(rate)(a, V, v, t, p), kin = PORT_T(rate)(a, V, v, p, t);
                if (!bnd[t] && !(mtc && bnd[p])) At[t * P + t] -= kgo;
                Al[t * P + t] -= kgo;
                if (!bnd[t] && !bnd[p]) At[t * P + p] += kin;
                Al[t * P + p] += kin;
            }
        }
        for (int i = 0; i < P * P; ++i) {
            At[i] *= (double)dt;
            Al[i] *= (double)dt;
        }
        port_expm1_phi1(P, At, Ft, Xt);
        port_expm1_phi1(P, Al, Fl, Xl);
        for (int t = 0; t < P; ++t) {
            if (!on[t]) continue;
            double x = rx[t], y = ry[t], z = rz[t];
            for (int p = 0; p < P; ++p) {
                x += Ft[t * P + p] * (double)rx[p];
                y += Ft[t * P + p] * (double)ry[p];
                z += Fl[t * P + p] * (double)rz[p] + (double)dt * Xl[t * P + p] * b[p];
            }
            MX[IDX(t)] = (REAL)x;
            MY[IDX(t)] = (REAL)y;
            MZ[IDX(t)] = (REAL)z;
        }
        return;
    }

    if (a->model == MRL_PORT_ME || a->model == MRL_PORT_GM) {
        REAL px[MRL_PORT_MAX_POOL], py[MRL_PORT_MAX_POOL], pz[MRL_PORT_MAX_POOL];
        for (int t = 0; t < P; ++t) {
            px[t] = MX[IDX(t)];
            py[t] = MY[IDX(t)];
            pz[t] = MZ[IDX(t)];
        }
        for (int t = 0; t < P; ++t) {
            REAL T1 = a->t1[PIDX(t)], T2 = a->t2[PIDX(t)], rho = a->rho[PIDX(t)];
            if (T2 == 0 || T1 == 0 || rho == 0) continue;
            int bound = (a->model == MRL_PORT_GM) && ((int)a->type_flag[t] == 1);
            int kind = (a->model == MRL_PORT_GM) ? (int)a->type_flag[t] : 0;
            if (kind != 0 && kind != 1) continue; /* unknown pool kind: left as is */
            REAL x = px[t], y = py[t], z = pz[t];
            if (!bound) {
                PORT_T(rotate)(&x, &y, &z, DW(t), st, tx, gyro, mg, pe, rf_sum);
            } else if (rf_sum != 0) {
                REAL w = PORT_T(bound_w)(st, tx, gyro, mg, db0, T2);
                z = z * REXP((REAL)(-w * dt));
            }
            REAL e1 = REXP((REAL)(-dt / T1));
            REAL m0 = (rho * ((REAL)1 - e1)) / (REAL)S;
            REAL kout = 1, kx = 0, ky = 0, kz = 0;
            for (int p = 0; p < P; ++p) {
                if (a->model == MRL_PORT_GM && p == t) continue;
                /* ME: channel t*P+p is the rate t->p; GM: channel p*P+t */
                REAL kgo = a->model == MRL_PORT_ME ? a->k[(long)(t * P + p) * V + v] : a->k[(long)(p * P + t) * V + v];
                REAL kin = a->model == MRL_PORT_ME ? a->k[(long)(p * P + t) * V + v] : a->k[(long)(t * P + p) * V + v];
                if (kgo != 0) kout *= REXP((REAL)(-dt * kgo));
                if (kin != 0) {
                    REAL f = (REAL)1 - REXP((REAL)(-dt * kin));
                    if (!bound) {
                        kx += f * px[p];
                        ky += f * py[p];
                    }
                    kz += f * pz[p];
                }
            }
            if (!bound) {
                REAL e2 = REXP((REAL)(-dt / T2));
                x *= e2;
                y *= e2;
                MX[IDX(t)] = x * kout + kx;
                MY[IDX(t)] = y * kout + ky;
            }
            z *= e1;
            MZ[IDX(t)] = z * kout + kz + m0;
        }
        return;
    }

    /* MT and CEST: pool 0 free water, pool 1 bound (MT) pool */
    {
        REAL T1 = a->t1[PIDX(0)], T2 = a->t2[PIDX(0)], rho = a->rho[PIDX(0)];
        if (T2 == 0 || T1 == 0 || rho == 0) return;
        REAL T1b = a->t1[PIDX(1)], T2b = a->t2[PIDX(1)], rhob = a->rho[PIDX(1)];
        REAL K12, K21;
        if (a->model == MRL_PORT_MT) {
            K12 = a->k[1L * V + v];
            K21 = a->k[2L * V + v];
        } else {
            K12 = a->k[0L * V + v];
            K21 = a->k[(long)(P - 1) * V + v];
        }
        REAL x = MX[IDX(0)], y = MY[IDX(0)], z = MZ[IDX(0)];
        REAL zb = MZ[IDX(1)];
        REAL cx[MRL_PORT_MAX_POOL], cy[MRL_PORT_MAX_POOL], cz[MRL_PORT_MAX_POOL];
        for (int t = 2; t < P; ++t) {
            cx[t] = MX[IDX(t)];
            cy[t] = MY[IDX(t)];
            cz[t] = MZ[IDX(t)];
        }
        const REAL x0 = x, y0 = y, z0 = z, zb0 = zb;
        PORT_T(rotate)(&x, &y, &z, DW(0), st, tx, gyro, mg, pe, rf_sum);
        REAL e2 = REXP((REAL)(-dt / T2));
        REAL e1k = REXP((REAL)(-dt / T1 - dt * K12));
        REAL m0 = (rho * ((REAL)1 - REXP((REAL)(-dt / T1)))) / (REAL)S;
        REAL ek = (REAL)1 - REXP((REAL)(-dt * K21));
        if (a->model == MRL_PORT_MT) {
            x = x * e2;
            y = y * e2;
            z = z * e1k + m0 + zb0 * ek;
        } else {
            REAL kout = 1, kx = 0, ky = 0, kz = 0;
            for (int t = 2; t < P; ++t) {
                REAL kgo = a->k[(long)(t - 1) * V + v];
                REAL kin = a->k[(long)(t + P - 2) * V + v];
                if (kgo != 0) kout *= REXP((REAL)(-dt * kgo));
                if (kin != 0) {
                    REAL f = (REAL)1 - REXP((REAL)(-dt * kin));
                    kx += f * cx[t];
                    ky += f * cy[t];
                    kz += f * cz[t];
                }
            }
            x = x * e2 * kout + kx;
            y = y * e2 * kout + ky;
            z = z * e1k * kout + kz + zb0 * ek + m0;
            /* CEST pools exchange with the free pool's state at the step start */
            for (int t = 2; t < P; ++t) {
                REAL T1c = a->t1[PIDX(t)], T2c = a->t2[PIDX(t)], rhoc = a->rho[PIDX(t)];
                REAL X = cx[t], Yv = cy[t], Z = cz[t];
                PORT_T(rotate)(&X, &Yv, &Z, DW(t), st, tx, gyro, mg, pe, rf_sum);
                REAL c2 = REXP((REAL)(-dt / T2c));
                REAL c1 = REXP((REAL)(-dt / T1c));
                REAL cm0 = (rhoc * ((REAL)1 - c1)) / (REAL)S;
                X *= c2;
                Yv *= c2;
                Z *= c1;
                REAL ko = 1, ix = 0, iy = 0, iz = 0;
                REAL kgo = a->k[(long)(t + P - 2) * V + v];
                REAL kin = a->k[(long)(t - 1) * V + v];
                if (kgo != 0) ko = REXP((REAL)(-dt * kgo));
                if (kin != 0) {
                    REAL f = (REAL)1 - REXP((REAL)(-dt * kin));
                    ix = f * x0;
                    iy = f * y0;
                    iz = f * z0;
                }
                MX[IDX(t)] = X * ko + ix;
                MY[IDX(t)] = Yv * ko + iy;
                MZ[IDX(t)] = Z * ko + iz + cm0;
            }
        }
        /* bound pool: saturation, then relaxation and exchange with the free
         * pool's Mz of the previous step */
        REAL bz = zb;
        if (rf_sum != 0) {
            REAL w = PORT_T(bound_w)(st, tx, gyro, mg, db0, T2b);
            bz = zb * REXP((REAL)(-w * dt));
        }
        REAL e1b = REXP((REAL)(-dt / T1b - dt * K21));
        REAL m0b = (rhob * ((REAL)1 - REXP((REAL)(-dt / T1b)))) / (REAL)S;
        REAL ekb = (REAL)1 - REXP((REAL)(-dt * K12));
        MZ[IDX(1)] = bz * e1b + m0b + z0 * ekb;
        MX[IDX(0)] = x;
        MY[IDX(0)] = y;
        MZ[IDX(0)] = z;
    }
#undef IDX
#undef PIDX
#undef DW
}

/* Is pool t of voxel v sampled by the receiver, and is the voxel active? */
static int PORT_T(sampled)(const mrl_port_args *a, long V, int v, int t) {
    if (a->model == MRL_PORT_NORMAL || a->model == MRL_PORT_ME || a->model == MRL_PORT_GM) {
        if (a->model == MRL_PORT_GM && (int)a->type_flag[t] != 0) return 0;
        return 1;
    }
    return t == 0;
}

int PORT_FN(const mrl_port_args *a, long long *steps_done) {
    if (!a || a->type_num < 1 || a->type_num > MRL_PORT_MAX_POOL || a->tx_num < 1 ||
        a->tx_num > MRL_PORT_MAX_TX || a->rx_num < 1 || a->spin_num < 1)
        return -1;
    if ((a->model == MRL_PORT_MT && a->type_num != 2) || (a->model == MRL_PORT_CEST && a->type_num < 2))
        return -1;
    if (a->exact) { /* ME, MT, CEST, or GM with free (TypeFlag 0) and bound (1) pools */
        if (a->model == MRL_PORT_NORMAL) return -1;
        for (int t = 0; a->model == MRL_PORT_GM && t < a->type_num; ++t)
            if ((int)a->type_flag[t] != 0 && (int)a->type_flag[t] != 1) return -1;
    }
    const long V = (long)a->ny * a->nx * a->nz;
    const int P = a->type_num, S = a->spin_num, TX = a->tx_num, RX = a->rx_num, A = a->signal_num;
    const long N = (long)P * S * V;
    REAL *MX = (REAL *)malloc(sizeof(REAL) * N), *MY = (REAL *)malloc(sizeof(REAL) * N),
         *MZ = (REAL *)malloc(sizeof(REAL) * N);
    for (long i = 0; i < N; ++i) {
        MX[i] = a->mx[i];
        MY[i] = a->my[i];
        MZ[i] = a->mz[i];
    }
    const REAL gyro = (REAL)a->gyro;
    int nthreads = 1;
#ifdef _OPENMP
    nthreads = a->threads > 0 ? a->threads : omp_get_max_threads();
#endif
    const int nval = P * RX * 2;
    double *part = (double *)calloc((size_t)nthreads * nval, sizeof(double));

    /* VVar state (DoPreScan.m:517-548) */
    double rfAmp[MRL_PORT_MAX_TX] = {0}, rfPhase[MRL_PORT_MAX_TX] = {0}, rfFreq[MRL_PORT_MAX_TX] = {0};
    double GzAmp = 0, GyAmp = 0, GxAmp = 0, ADC = 0, Ext = 0, KzT = 0, KyT = 0, KxT = 0;
    int utsi = 0, rfi = 0, Gzi = 0, Gyi = 0, Gxi = 0, ADCi = 0, Exti = 0, signali = 0;
    long long done = 0;
    int i = 0;
    const int MaxStep = a->n_ts;
    while (i < MaxStep - 1) {
        /* merge the flags of all entries sharing one time point (DoScanAtCPU.cpp:247-284) */
        double flag[6] = {0, 0, 0, 0, 0, 0};
        if (a->ts[i] != a->ts[i + 1]) {
            for (int f = 0; f < 6; ++f) flag[f] += a->flags[(long)i * 6 + f];
            i++;
        } else {
            for (int f = 0; f < 6; ++f) flag[f] += a->flags[(long)i * 6 + f];
            while (a->ts[i] == a->ts[i + 1]) {
                for (int f = 0; f < 6; ++f) flag[f] += a->flags[(long)(i + 1) * 6 + f];
                i++;
                if (i == MaxStep - 1) break;
            }
            i++;
        }
        const int un = a->n_uts;
        const int nxt = utsi + 1 < un - 1 ? utsi + 1 : un - 1;
        const double dt = a->uts[nxt] - a->uts[utsi];
        utsi = nxt;
        /* sample-and-hold: the smaller-magnitude end of each interval (:298-354) */
        if (flag[0] >= 1) {
            for (int j = 0; j < flag[0]; ++j) {
                double coil = a->rf_coil[rfi];
                int txi = (int)coil;
                for (int s2 = rfi + 1; s2 < a->n_rf; ++s2) {
                    if (coil == a->rf_coil[s2]) {
                        if (txi >= 1 && txi <= TX) {
                            rfAmp[txi - 1] = fabs(a->rf_amp[rfi]) <= fabs(a->rf_amp[s2]) ? a->rf_amp[rfi] : a->rf_amp[s2];
                            rfPhase[txi - 1] = fabs(a->rf_phase[rfi]) <= fabs(a->rf_phase[s2]) ? a->rf_phase[rfi] : a->rf_phase[s2];
                            rfFreq[txi - 1] = fabs(a->rf_freq[rfi]) <= fabs(a->rf_freq[s2]) ? a->rf_freq[rfi] : a->rf_freq[s2];
                        }
                        break;
                    }
                }
                rfi++;
            }
        }
#define HOLD(flagv, line, n, idx, out)                                                   \
    if ((flagv) == 1) {                                                                  \
        int nn = (idx) + 1 < (n)-1 ? (idx) + 1 : (n)-1;                                  \
        out = fabs((line)[idx]) <= fabs((line)[nn]) ? (line)[idx] : (line)[(idx) + 1];   \
        (idx)++;                                                                         \
    }
        HOLD(flag[1], a->gz, a->n_gz, Gzi, GzAmp)
        HOLD(flag[2], a->gy, a->n_gy, Gyi, GyAmp)
        HOLD(flag[3], a->gx, a->n_gx, Gxi, GxAmp)
#undef HOLD
        ADC = 0;
        if (flag[4] == 1) {
            ADC = a->adc[ADCi];
            ADCi++;
        }
        if (flag[5] == 1) {
            Ext = a->ext[Exti];
            if (Ext != 0 && a->ext_cb) {
                for (long q = 0; q < N; ++q) {
                    a->mx[q] = (float)MX[q];
                    a->my[q] = (float)MY[q];
                    a->mz[q] = (float)MZ[q];
                }
                if (a->ext_cb(a->ext_user, Ext) != 0) {
                    free(MX), free(MY), free(MZ), free(part);
                    return -2;
                }
                for (long q = 0; q < N; ++q) {
                    MX[q] = a->mx[q];
                    MY[q] = a->my[q];
                    MZ[q] = a->mz[q];
                }
            }
            Exti++;
        }
        if (flag[0] + flag[1] + flag[2] + flag[3] + flag[4] + flag[5] == 0) {
            for (int c = 0; c < TX; ++c) rfAmp[c] = rfPhase[c] = rfFreq[c] = 0;
            GzAmp = GyAmp = GxAmp = 0;
            ADC = 0;
            Ext = 0;
        }
        if (dt < 0 && a->run_mode == 1 && a->mxs) { /* TR boundary (DoScanAtCPU.cpp:431-436) */
            for (long q = 0; q < N; ++q) {
                a->mxs[(long)utsi * N + q] = (float)MX[q];
                a->mys[(long)utsi * N + q] = (float)MY[q];
                a->mzs[(long)utsi * N + q] = (float)MZ[q];
            }
            if (a->muts && utsi > 0) a->muts[utsi] = a->muts[utsi - 1];
        }
        if (dt <= 0) continue; /* end of a time point, or TR boundary */
        if (a->max_steps >= 0 && done >= a->max_steps) break;

        PORT_T(step) st;
        st.dt = (REAL)dt;
        REAL rf_sum = 0;
        for (int c = 0; c < TX; ++c) {
            REAL amp = (REAL)rfAmp[c], ph = (REAL)rfPhase[c];
            if (amp < 0) { /* negative amplitude: flip the phase (BlochKernel.h:62-65) */
                amp = (REAL)fabs((double)amp);
                ph = (REAL)((double)ph + PI);
            }
            st.amp[c] = amp;
            st.phase[c] = ph;
            st.freq[c] = (REAL)rfFreq[c];
            rf_sum += (REAL)fabs((double)(REAL)rfAmp[c]);
        }
        st.gz = (REAL)GzAmp;
        st.gy = (REAL)GyAmp;
        st.gx = (REAL)GxAmp;
        st.adc = ADC == 1;
        if (a->steps_out && done < a->steps_cap) {
            double *r = a->steps_out + done * (10 + 3 * (TX - 1));
            r[0] = dt, r[1] = GzAmp, r[2] = GyAmp, r[3] = GxAmp;
            r[4] = (double)st.amp[0], r[5] = (double)st.phase[0], r[6] = (double)st.freq[0];
            r[7] = (double)rf_sum, r[8] = st.adc ? 1.0 : 0.0, r[9] = (double)signali;
            for (int c = 1; c < TX; ++c)
                r[10 + 3 * (c - 1)] = (double)st.amp[c], r[11 + 3 * (c - 1)] = (double)st.phase[c],
                r[12 + 3 * (c - 1)] = (double)st.freq[c];
        }

        /* receive before this step's rotation (DoScanAtCPU.cpp:445-491) */
        if (st.adc && signali < A) {
            const REAL cr = (REAL)cos(-a->rf_ref), sr = (REAL)sin(-a->rf_ref);
            memset(part, 0, sizeof(double) * (size_t)nthreads * nval);
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(static)
#endif
            for (long v = 0; v < V; ++v) {
                int tid = 0;
#ifdef _OPENMP
                tid = omp_get_thread_num();
#endif
                double *pp = part + (size_t)tid * nval;
                for (int t = 0; t < P; ++t) {
                    if (!PORT_T(sampled)(a, V, (int)v, t)) continue;
                    for (int s = 0; s < S; ++s) {
                        long idx = (long)t * S * V + (long)s * V + v;
                        REAL mx = MX[idx], my = MY[idx];
                        for (int c = 0; c < RX; ++c) {
                            REAL b1, b3;
                            if (a->rx_default == 0) {
                                REAL rx = a->rx_x[(long)c * V + v], ry = a->rx_y[(long)c * V + v];
                                b1 = mx * rx + my * ry;
                                b3 = -mx * ry + my * rx;
                            } else {
                                b1 = mx;
                                b3 = my;
                            }
                            if (a->rf_ref != 0) {
                                REAL n1 = b1 * cr + b3 * -sr;
                                REAL n3 = b1 * sr + b3 * cr;
                                b1 = n1;
                                b3 = n3;
                            }
                            pp[(t * RX + c) * 2 + 0] += (double)b1;
                            pp[(t * RX + c) * 2 + 1] += (double)b3;
                        }
                    }
                }
            }
            for (int th = 0; th < nthreads; ++th)
                for (int t = 0; t < P; ++t)
                    for (int c = 0; c < RX; ++c) {
                        a->sx[(long)t * RX * A + (long)c * A + signali] += part[(size_t)th * nval + (t * RX + c) * 2];
                        a->sy[(long)t * RX * A + (long)c * A + signali] += part[(size_t)th * nval + (t * RX + c) * 2 + 1];
                    }
        }

#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(static)
#endif
        for (long v = 0; v < V; ++v)
            for (int s = 0; s < S; ++s) PORT_T(update)(a, MX, MY, MZ, V, (int)v, s, &st, rf_sum, gyro);
        done++;

        if (st.adc) {
            if (signali < A) {
                a->kz[signali] += KzT;
                a->ky[signali] += KyT;
                a->kx[signali] += KxT;
            }
            signali++;
        }
        KzT += GzAmp * dt * (a->gyro / (2 * PI));
        KyT += GyAmp * dt * (a->gyro / (2 * PI));
        KxT += GxAmp * dt * (a->gyro / (2 * PI));
        if (a->run_mode == 1 && a->mxs) { /* DoScanAtCPU.cpp:544-552 */
            for (long q = 0; q < N; ++q) {
                a->mxs[(long)utsi * N + q] = (float)MX[q];
                a->mys[(long)utsi * N + q] = (float)MY[q];
                a->mzs[(long)utsi * N + q] = (float)MZ[q];
            }
            if (a->muts && utsi > 0) a->muts[utsi] = a->muts[utsi - 1] + dt;
        }
    }
    for (long q = 0; q < N; ++q) {
        a->mx[q] = (float)MX[q];
        a->my[q] = (float)MY[q];
        a->mz[q] = (float)MZ[q];
    }
    free(MX), free(MY), free(MZ), free(part);
    if (steps_done) *steps_done = done;
    return 0;
}

#undef RSIN
#undef RCOS
