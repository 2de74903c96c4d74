/* cpu_port.c -- multi-threaded FP64 C restatement of the reference's plain 3D
 * solve for the CPU baseline (oracle: test and measurement infrastructure only;
 * the product never links it).
 *
 * It restates, on the host cores:
 *   - lap3D, the 27-point nodal operator (laplacian.py:898-1026), in the form of
 *     oracle/nodal3d.py's lap3d: unknowns are the inner nodes in C order (z
 *     fastest), a periodic axis wraps with the duplicated seam (wrap distance
 *     n-1, the neighbour of node 0 is node n-2 and of node n-1 is node 1), a wall
 *     axis zeroes the hplus of its outer cell planes (laplacian.py:933-965);
 *     four-edge differences per cell (:968-985), cell coefficients times them
 *     (:987-1015), the node sums, the 1/16 factor, the Coriolis cross terms,
 *     hcenter * p and the diag_inv scaling (:1017-1024);
 *   - scipy.sparse.linalg.bicgstab as the reference calls it
 *     (second_projection.py:230): x0 = 0, the legacy exit ||b|| <= tol -> x = 0,
 *     atol = tol * ||b||, scipy's loop (rho, rho/omega breakdown at eps^2,
 *     early exit on ||s||, convergence on ||r|| at the top of each iteration).
 *
 * The reference runs its Numba kernels on one thread and its inner products
 * through BLAS threads; this port runs every loop with OpenMP over the x axis so
 * that the baseline uses all the host cores it is given.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    int nx, ny, nz;
    int x_wall, y_wall, z_wall;
    double dx, dy, dz, corrf;
    const double *hplusx, *hplusy, *hplusz;   /* (nx+1)(ny+1)(nz+1) cells, C order */
    const double *hcenter;                    /* nodes, may be NULL (== 0) */
    const double *diag_inv;                   /* nodes */
} port_op3d;

int port_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* padded-node index along an axis of n inner nodes: -1 -> n-2, n -> 1 */
static inline int wrap(int i, int n) { return i < 0 ? n - 2 : (i >= n ? 1 : i); }

typedef struct {
    port_op3d op;
    double *hx, *hy, *hz;        /* wall-zeroed copies */
    double *fx, *fy, *fz;        /* cell fluxes h_d * S_d p */
    double *cxz, *czx;           /* Coriolis cross fluxes hx * S_z p, hz * S_x p */
    int cross;
} lap3;

static void lap3_free(lap3 *L) {
    free(L->hx); free(L->hy); free(L->hz);
    free(L->fx); free(L->fy); free(L->fz);
    free(L->cxz); free(L->czx);
}

static int lap3_init(lap3 *L, const port_op3d *op) {
    memset(L, 0, sizeof(*L));
    L->op = *op;
    const int cx = op->nx + 1, cy = op->ny + 1, cz = op->nz + 1;
    const size_t nc = (size_t)cx * cy * cz;
    L->cross = op->corrf != 0.0;
    L->hx = malloc(nc * sizeof(double)); L->hy = malloc(nc * sizeof(double)); L->hz = malloc(nc * sizeof(double));
    L->fx = malloc(nc * sizeof(double)); L->fy = malloc(nc * sizeof(double)); L->fz = malloc(nc * sizeof(double));
    if (L->cross) { L->cxz = malloc(nc * sizeof(double)); L->czx = malloc(nc * sizeof(double)); }
    if (!L->hx || !L->hy || !L->hz || !L->fx || !L->fy || !L->fz || (L->cross && (!L->cxz || !L->czx))) {
        lap3_free(L);
        return -1;
    }
#pragma omp parallel for schedule(static)
    for (int I = 0; I < cx; ++I)
        for (int J = 0; J < cy; ++J)
            for (int K = 0; K < cz; ++K) {
                const size_t c = ((size_t)I * cy + J) * cz + K;
                const int wall = (op->x_wall && (I == 0 || I == cx - 1)) || (op->y_wall && (J == 0 || J == cy - 1)) ||
                                 (op->z_wall && (K == 0 || K == cz - 1));
                L->hx[c] = wall ? 0.0 : op->hplusx[c];
                L->hy[c] = wall ? 0.0 : op->hplusy[c];
                L->hz[c] = wall ? 0.0 : op->hplusz[c];
            }
    return 0;
}

/* y = lap3D(p) on the inner nodes */
static void lap3_apply(const lap3 *L, const double *p, double *y) {
    const int nx = L->op.nx, ny = L->op.ny, nz = L->op.nz;
    const int cy = ny + 1, cz = nz + 1;
#define P(i, j, k) p[((size_t)wrap(i, nx) * ny + wrap(j, ny)) * nz + wrap(k, nz)]
#pragma omp parallel for schedule(static)
    for (int I = 0; I <= nx; ++I)              /* cell I lies between padded nodes I-1 and I */
        for (int J = 0; J <= ny; ++J)
            for (int K = 0; K <= nz; ++K) {
                const int i0 = I - 1, j0 = J - 1, k0 = K - 1;
                const double p000 = P(i0, j0, k0), p001 = P(i0, j0, k0 + 1), p010 = P(i0, j0 + 1, k0),
                             p011 = P(i0, j0 + 1, k0 + 1), p100 = P(i0 + 1, j0, k0), p101 = P(i0 + 1, j0, k0 + 1),
                             p110 = P(i0 + 1, j0 + 1, k0), p111 = P(i0 + 1, j0 + 1, k0 + 1);
                const double sx = (p100 - p000) + (p101 - p001) + (p110 - p010) + (p111 - p011);
                const double sy = (p010 - p000) + (p110 - p100) + (p011 - p001) + (p111 - p101);
                const double sz = (p001 - p000) + (p011 - p010) + (p101 - p100) + (p111 - p110);
                const size_t c = ((size_t)I * cy + J) * cz + K;
                L->fx[c] = L->hx[c] * sx;
                L->fy[c] = L->hy[c] * sy;
                L->fz[c] = L->hz[c] * sz;
                if (L->cross) { L->cxz[c] = L->hx[c] * sz; L->czx[c] = L->hz[c] * sx; }
            }
#undef P
    const double co = 1.0 / 16.0;
    const double ox2 = 1.0 / (L->op.dx * L->op.dx), oy2 = 1.0 / (L->op.dy * L->op.dy), oz2 = 1.0 / (L->op.dz * L->op.dz);
    const double oxz = L->op.corrf / (L->op.dx * L->op.dz);
#define C(a, I, J, K) (a)[((size_t)(I) * cy + (J)) * cz + (K)]
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                /* node (i, j, k) sits between cells i and i+1 (etc.) */
                const double xm = C(L->fx, i, j, k) + C(L->fx, i, j, k + 1) + C(L->fx, i, j + 1, k) + C(L->fx, i, j + 1, k + 1);
                const double xp = C(L->fx, i + 1, j, k) + C(L->fx, i + 1, j, k + 1) + C(L->fx, i + 1, j + 1, k) +
                                  C(L->fx, i + 1, j + 1, k + 1);
                const double ym = C(L->fy, i, j, k) + C(L->fy, i, j, k + 1) + C(L->fy, i + 1, j, k) + C(L->fy, i + 1, j, k + 1);
                const double yp = C(L->fy, i, j + 1, k) + C(L->fy, i, j + 1, k + 1) + C(L->fy, i + 1, j + 1, k) +
                                  C(L->fy, i + 1, j + 1, k + 1);
                const double zm = C(L->fz, i, j, k) + C(L->fz, i, j + 1, k) + C(L->fz, i + 1, j, k) + C(L->fz, i + 1, j + 1, k);
                const double zp = C(L->fz, i, j, k + 1) + C(L->fz, i, j + 1, k + 1) + C(L->fz, i + 1, j, k + 1) +
                                  C(L->fz, i + 1, j + 1, k + 1);
                double v = ox2 * co * (xp - xm) + oy2 * co * (yp - ym) + oz2 * co * (zp - zm);
                if (L->cross) {
                    const double hxzm = C(L->cxz, i, j, k) + C(L->cxz, i, j, k + 1) + C(L->cxz, i, j + 1, k) +
                                        C(L->cxz, i, j + 1, k + 1);
                    const double hxzp = C(L->cxz, i + 1, j, k) + C(L->cxz, i + 1, j, k + 1) + C(L->cxz, i + 1, j + 1, k) +
                                        C(L->cxz, i + 1, j + 1, k + 1);
                    const double hzxm = C(L->czx, i, j, k) + C(L->czx, i, j + 1, k) + C(L->czx, i + 1, j, k) +
                                        C(L->czx, i + 1, j + 1, k);
                    const double hzxp = C(L->czx, i, j, k + 1) + C(L->czx, i, j + 1, k + 1) + C(L->czx, i + 1, j, k + 1) +
                                        C(L->czx, i + 1, j + 1, k + 1);
                    v += oxz * co * (hxzp - hxzm) - oxz * co * (hzxp - hzxm);
                }
                const size_t g = ((size_t)i * ny + j) * nz + k;
                if (L->op.hcenter) v += L->op.hcenter[g] * p[g];
                y[g] = v * L->op.diag_inv[g];
            }
#undef C
}

int port_lap3d(const port_op3d *op, const double *p, double *y) {
    lap3 L;
    if (lap3_init(&L, op) != 0) return -1;
    lap3_apply(&L, p, y);
    lap3_free(&L);
    return 0;
}

static double dot(const double *a, const double *b, long long n) {
    double s = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : s)
    for (long long g = 0; g < n; ++g) s += a[g] * b[g];
    return s;
}

/* Plain FP64 BiCGStab in scipy's control flow; stops after maxiter iterations.
 * Returns scipy's info (0 converged, maxiter, -10 rho breakdown, -11 omega
 * breakdown); *iters = iterations done, *relres = ||b - A x|| / ||b|| of the
 * recursive residual. */
int port_bicgstab3d(const port_op3d *op, const double *b, double *x, double tol, int maxiter, int *iters,
                    double *relres) {
    const long long n = (long long)op->nx * op->ny * op->nz;
    lap3 L;
    if (lap3_init(&L, op) != 0) return -100;
    double *r = malloc(n * sizeof(double)), *rt = malloc(n * sizeof(double)), *p = malloc(n * sizeof(double)),
           *v = malloc(n * sizeof(double)), *t = malloc(n * sizeof(double));
    int info = -100;
    *iters = 0;
    if (!r || !rt || !p || !v || !t) goto done;
    const double bnrm = sqrt(dot(b, b, n));
    memset(x, 0, n * sizeof(double));
    *relres = 0.0;
    if (bnrm <= tol) { info = 0; goto done; }          /* scipy 1.7 legacy exit, x = 0 */
    const double atol = tol * bnrm, eps = 2.220446049250313e-16, rhotol = eps * eps;
    memcpy(r, b, n * sizeof(double));
    memcpy(rt, b, n * sizeof(double));
    double rho_prev = 0.0, omega = 0.0, alpha = 0.0;
    info = maxiter;
    for (int it = 0; it < maxiter; ++it) {
        const double rn = sqrt(dot(r, r, n));
        *relres = rn / bnrm;
        if (rn < atol) { info = 0; break; }
        const double rho = dot(rt, r, n);
        if (fabs(rho) < rhotol) { info = -10; break; }
        if (it > 0) {
            if (fabs(omega) < rhotol) { info = -11; break; }
            const double beta = (rho / rho_prev) * (alpha / omega);
#pragma omp parallel for schedule(static)
            for (long long g = 0; g < n; ++g) p[g] = (p[g] - omega * v[g]) * beta + r[g];
        } else {
            memcpy(p, r, n * sizeof(double));
        }
        lap3_apply(&L, p, v);
        const double rv = dot(rt, v, n);
        if (rv == 0.0) { info = -11; break; }
        alpha = rho / rv;
#pragma omp parallel for schedule(static)
        for (long long g = 0; g < n; ++g) r[g] -= alpha * v[g];      /* s */
        const double sn = sqrt(dot(r, r, n));
        if (sn < atol) {
#pragma omp parallel for schedule(static)
            for (long long g = 0; g < n; ++g) x[g] += alpha * p[g];
            *iters = it + 1;
            *relres = sn / bnrm;
            info = 0;
            break;
        }
        lap3_apply(&L, r, t);
        omega = dot(t, r, n) / dot(t, t, n);
#pragma omp parallel for schedule(static)
        for (long long g = 0; g < n; ++g) {
            x[g] += alpha * p[g] + omega * r[g];
            r[g] -= omega * t[g];
        }
        rho_prev = rho;
        *iters = it + 1;
    }
    if (info == maxiter) *relres = sqrt(dot(r, r, n)) / bnrm;
done:
    free(r); free(rt); free(p); free(v); free(t);
    lap3_free(&L);
    return info;
}
