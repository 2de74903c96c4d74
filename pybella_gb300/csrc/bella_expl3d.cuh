// bella_expl3d.cuh -- arithmetic of the explicit parts of the 3D projection
// (second_projection.py:22-92), one cell or node at a time.
//
// __host__ __device__ functions: the kernels of bella_expl3d.cu run them one thread
// per item, and tests/expl3d_host.cpp runs the same source on the CPU against the
// oracle.  Cells (icx, icy, icz) and nodes (icx+1, icy+1, icz+1) in the reference's
// C order over (x, y, z), two ghost layers; node.isc = (icx-1, icy-1, icz-1).
#pragma once
#include <math.h>

#ifdef __CUDACC__
#define BELLA_HD __host__ __device__ __forceinline__
#else
#define BELLA_HD inline
#endif

namespace bella {

struct Expl3Geom {
    int icx, icy, icz;
    int bc[3];                       // 0 periodic, 1 wall
    double dx, dy, dz, dt;
    double Msq, g, gamm, nonhydro, compressibility;
    double cor[3];                   // ud.coriolis_strength
    double wind[3];                  // ud.u_wind_speed, v_wind_speed, w_wind_speed
    double xsign;                    // divergence x term: -1 as divergence_nodes' 3D branch, +1 as its 2D branch
    int is_ArakawaKonor;
};

struct Expl3Fields {                 // rho, rhou, rhov, rhow, rhoY, rhoX
    double *f[6];
};

BELLA_HD long long e3_cell(const Expl3Geom &G, int i, int j, int k) {
    return ((long long)i * G.icy + j) * G.icz + k;
}
BELLA_HD long long e3_node(const Expl3Geom &G, int i, int j, int k) {
    return ((long long)i * (G.icy + 1) + j) * (G.icz + 1) + k;
}
BELLA_HD long long e3_isc(const Expl3Geom &G, int a, int b, int c) {
    return ((long long)a * (G.icy - 1) + b) * (G.icz - 1) + c;
}

// euler_backward_non_advective_expl_part (second_projection.py:77-92) on cell e, before
// its boundary data: buoyancy into rhov, background wind off, the implicit Coriolis /
// buoyancy inverse (multiply_inverse_coriolis, :604-646), background wind on
BELLA_HD void e3_expl_part_cell(const Expl3Geom &G, long long e, int j, const double *S0n, const Expl3Fields &F) {
    double *rho = F.f[0], *rhou = F.f[1], *rhov = F.f[2], *rhow = F.f[3], *rhoY = F.f[4], *rhoX = F.f[5];
    const double dbuoy = rhoY[e] * (rhoX[e] / rho[e]);
    double U = rhou[e], V = (G.nonhydro * rhov[e]) - G.dt * (G.g / G.Msq) * dbuoy, W = rhow[e];
    U = U + -1.0 * G.wind[0] * rho[e];
    V = V + -1.0 * G.wind[1] * rho[e];
    W = W + -1.0 * G.wind[2] * rho[e];
    const double nonhydro = G.nonhydro;
    const double wh1 = G.dt * G.cor[0], wv = G.dt * G.cor[1], wh2 = G.dt * G.cor[2];
    const double strat = (S0n[j + 1] - S0n[j]) / G.dy;
    const double Y = rhoY[e] / rho[e];
    const double nu = -(G.dt * G.dt) * (G.g / G.Msq) * strat * Y;
    const double denom = 1.0 / (wh1 * wh1 + wh2 * wh2 + (nu + nonhydro) * (wv * wv + 1.0));
    const double uu = (wh1 * wh1 + nu + nonhydro), uv = nonhydro * (wh1 * wv + wh2),
                 uw = (wh1 * wh2 - (nu + nonhydro) * wv);
    const double vu = (wh1 * wv - wh2), vv = nonhydro * (1 + wv * wv), vw = (wh2 * wv + wh1);
    const double wu = (wh1 * wh2 + (nu + nonhydro) * wv), wvv = nonhydro * (wh2 * wv - wh1),
                 ww = (nu + nonhydro + wh2 * wh2);
    const double U2 = denom * (uu * U + uv * V + uw * W);
    const double V2 = denom * (vu * U + vv * V + vw * W);
    const double W2 = denom * (wu * U + wvv * V + ww * W);
    rhou[e] = U2 + 1.0 * G.wind[0] * rho[e];
    rhov[e] = V2 + 1.0 * G.wind[1] * rho[e];
    rhow[e] = W2 + 1.0 * G.wind[2] * rho[e];
}

// scale_wall_node_values (second_projection.py:433-474) on node.isc: the wall index of
// an earlier wall axis stays at row 1 for the later ones
BELLA_HD double e3_wall_scale(const Expl3Geom &G, int a, int b, int c, double f) {
    const int x[3] = {a, b, c}, n[3] = {G.icx - 1, G.icy - 1, G.icz - 1};
    double s = 1.0;
    for (int d = 0; d < 3; ++d) {
        if (!G.bc[d]) continue;
        for (int t = 0; t < 2; ++t) {
            const int row = t == 0 ? n[d] - 2 : 1;
            bool hit = true;
            for (int q = 0; q < 3; ++q) {
                if (q == d) hit = hit && x[q] == row;
                else if (q < d && G.bc[q]) hit = hit && x[q] == 1;
                else hit = hit && x[q] >= 2 && x[q] <= n[q] - 3;
            }
            if (hit) s *= f;
        }
    }
    return s;
}

// euler_forward_non_advective (second_projection.py:22-74), node part at node.isc
// (a, b, c): the divergence of the momenta (divergence_nodes' 3D branch with its
// x sign, :556-570; the y-wall ghost momenta already zeroed), wall rows doubled
// (:40), returned; dp = -dt * dpidP * div with dpidP = (gamma-1)/Msq times the
// 2x2x2 mean of rhoY^(gamma-2) (:45-47, :66)
BELLA_HD double e3_forward_node(const Expl3Geom &G, int a, int b, int c, const Expl3Fields &F, double *dp) {
    const double *rho = F.f[0], *rhou = F.f[1], *rhov = F.f[2], *rhow = F.f[3], *rhoY = F.f[4];
    double ux[2], vy[2], wz[2];
    for (int t = 0; t < 2; ++t) {
        auto q = [&](const double *m, int i, int j, int k) {
            const long long e = e3_cell(G, i, j, k);
            return m[e] * (rhoY[e] / rho[e]);
        };
        const double d0 = (q(rhou, a + 1, b, c + t) - q(rhou, a, b, c + t)) / G.dx;
        const double d1 = (q(rhou, a + 1, b + 1, c + t) - q(rhou, a, b + 1, c + t)) / G.dx;
        ux[t] = 0.5 * (d0 + d1);
        const double e0 = (q(rhov, a, b + 1, c + t) - q(rhov, a, b, c + t)) / G.dy;
        const double e1 = (q(rhov, a + 1, b + 1, c + t) - q(rhov, a + 1, b, c + t)) / G.dy;
        vy[t] = 0.5 * (e0 + e1);
        const double f0 = (q(rhow, a, b + t, c + 1) - q(rhow, a, b + t, c)) / G.dz;
        const double f1 = (q(rhow, a + 1, b + t, c + 1) - q(rhow, a + 1, b + t, c)) / G.dz;
        wz[t] = 0.5 * (f0 + f1);
    }
    const double Ux = (0.5 * G.xsign) * (ux[0] + ux[1]);
    const double Vy = 0.5 * (vy[0] + vy[1]);
    const double Wz = 0.5 * (wz[0] + wz[1]);
    double div = (Ux + Vy + Wz);
    div *= e3_wall_scale(G, a, b, c, 2.0);
    double s = 0.0;
    for (int q = 0; q < 8; ++q) s += pow(rhoY[e3_cell(G, a + (q >> 2), b + ((q >> 1) & 1), c + (q & 1))], G.gamm - 2.0);
    const double dpidP = ((G.gamm - 1.0) / G.Msq) * s / 8.0;
    *dp = -(G.dt * dpidP * div);
    return div;
}

// euler_forward_non_advective, cell part (:49-64): momenta from the pressure gradient
// of the old p2 (grad_nodes, :496-521), buoyancy and Coriolis of the background-wind
// deviations; rhoX from the background S0c and dS/dy
BELLA_HD void e3_forward_cell(const Expl3Geom &G, int i, int j, int k, const double *p2, const double *S0c,
                              const double *S0n, const Expl3Fields &F) {
    double *rho = F.f[0], *rhou = F.f[1], *rhov = F.f[2], *rhow = F.f[3], *rhoY = F.f[4], *rhoX = F.f[5];
    const long long e = e3_cell(G, i, j, k);
    double Dpx = 0.0, Dpy = 0.0, Dpz = 0.0;
    for (int q = 0; q < 8; ++q) {
        const int ox = q >> 2, oy = (q >> 1) & 1, oz = q & 1;
        const double v = p2[e3_node(G, i + ox, j + oy, k + oz)];
        Dpx = Dpx + (ox ? 1.0 : -1.0) * v;
        Dpy = Dpy + (oy ? 1.0 : -1.0) * v;
        Dpz = Dpz + (oz ? 1.0 : -1.0) * v;
    }
    Dpx = Dpx * (0.25 / G.dx);
    Dpy = Dpy * (0.25 / G.dy);
    Dpz = Dpz * (0.25 / G.dz);
    const double Ginv = G.gamm / (G.gamm - 1.0);
    const double rhoYovG = Ginv * rhoY[e];
    const double dbuoy = rhoY[e] * (rhoX[e] / rho[e]);
    const double drhou = rhou[e] - G.wind[0] * rho[e];
    const double drhov = rhov[e] - G.wind[1] * rho[e];
    const double drhow = rhow[e] - G.wind[2] * rho[e];
    const double v = rhov[e] / rho[e];
    const double ch1 = G.cor[0], cv = G.cor[1], ch2 = G.cor[2];
    rhou[e] = rhou[e] - G.dt * (rhoYovG * Dpx - ch2 * drhov + cv * drhow);
    rhov[e] = rhov[e] - G.dt * (rhoYovG * Dpy + (G.g / G.Msq) * dbuoy * G.nonhydro - ch1 * drhow + ch2 * drhou) *
                            (1 - G.is_ArakawaKonor);
    rhow[e] = rhow[e] - G.dt * (rhoYovG * Dpz - cv * drhou + ch1 * drhov) * 1;
    const double dSdy = (S0n[j + 1] - S0n[j]) / G.dy;
    rhoX[e] = (rho[e] * (rho[e] / rhoY[e] - S0c[e])) - G.dt * (v * dSdy) * rho[e];
}

}  // namespace bella

namespace bella {

// set_ghostnodes_p2 (boundary.py:296-369) along axis d for line l of nodes (the other
// two node axes in (x, y, z) order, outer first): periodic_plus_one or 'reflect'
BELLA_HD void e3_ghost_line(const Expl3Geom &G, int d, long long l, double *p) {
    const int nn[3] = {G.icx + 1, G.icy + 1, G.icz + 1};
    const int a1 = d == 0 ? 1 : 0, a2 = d == 2 ? 1 : 2;
    int x[3];
    x[a1] = (int)(l / nn[a2]);
    x[a2] = (int)(l - (long long)x[a1] * nn[a2]);
    const int n = nn[d];
    auto at = [&](int t) -> double & {
        x[d] = t;
        return p[((long long)x[0] * nn[1] + x[1]) * nn[2] + x[2]];
    };
    if (G.bc[d] == 0) {
        const double h0 = at(n - 5), h1 = at(n - 4), h2 = at(n - 3);
        const double t0 = at(2), t1 = at(3), t2 = at(4);
        at(0) = h0; at(1) = h1; at(2) = h2;
        at(n - 3) = t0; at(n - 2) = t1; at(n - 1) = t2;
    } else {
        at(0) = at(4);
        at(1) = at(3);
        at(n - 2) = at(n - 4);
        at(n - 1) = at(n - 5);
    }
}

}  // namespace bella
