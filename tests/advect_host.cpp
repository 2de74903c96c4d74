// Host build of the device advection arithmetic (pybella_gb300/csrc/bella_advect.cuh)
// for tests/test_advect_host.py: the same per-face, per-cell and per-line functions
// and the same sweep sequences the kernels of bella_advect.cu run, executed by loops,
// so their arithmetic and indexing are checked against the oracle without a GPU.
#include "../pybella_gb300/csrc/bella_advect.cuh"

using namespace bella;

namespace {

struct HostEx {
    AdvGeom G;
    AdvFields F;
    AdvFaces fl[3];
    const double *rhoY0, *strat_inv;
    double *pw;
    void bd(int s) {
        for (int l = 0; l < adv_nl(G, s); ++l) adv_bd_line(G, s, l, F, rhoY0, strat_inv);
    }
    void faces(int s, double lmbda) {
        for (int l = 0; l < adv_nl(G, s); ++l)
            for (int f = 1; f <= adv_ns(G, s) - 1; ++f) adv_face_flux(G, s, l, f, F, lmbda, fl[s]);
    }
    void update(int s, double lmbda) {
        for (int l = 0; l < adv_nl(G, s); ++l)
            for (int c = 0; c < adv_ns(G, s); ++c) adv_update_cell(G, s, l, c, F, fl[s], lmbda);
    }
    void mass() {
        for (int s = 0; s < G.nd; ++s)
            for (int l = 0; l < adv_nl(G, s); ++l)
                if (adv_inner_line(G, s, l))
                    for (int f = 1; f <= adv_ns(G, s) - 1; ++f) fl[s].f[4][adv_face(G, s, l, f)] = adv_mass(G, s, l, f, F);
    }
    void pwchi(double lmbda) {
        if (!pw) return;
        for (int l = 0; l < adv_nl(G, 1); ++l)
            for (int c = 0; c < adv_ns(G, 1); ++c)
                pw[adv_cell(G, 1, l, c)] = lmbda * (fl[1].f[5][adv_face(G, 1, l, c)] - fl[1].f[5][adv_face(G, 1, l, c + 1)]);
    }
};

// geo: nd, ic[3], walls[3] as ints; d[3], g, gamm as doubles; faces: nd arrays of 6 pointers
HostEx make(const int *geo, const double *dg, int comp, double **fields, double **faces, const double *rhoY0,
            const double *strat_inv, double *pw) {
    HostEx ex;
    ex.G.nd = geo[0];
    for (int a = 0; a < 3; ++a) {
        ex.G.ic[a] = geo[1 + a];
        ex.G.bc[a] = geo[4 + a];
        ex.G.d[a] = dg[a];
    }
    ex.G.g = dg[3]; ex.G.gamm = dg[4]; ex.G.is_compressible = comp;
    for (int q = 0; q < 6; ++q) {
        ex.F.f[q] = fields[q];
        for (int s = 0; s < 3; ++s) ex.fl[s].f[q] = s < ex.G.nd ? faces[6 * s + q] : nullptr;
    }
    ex.rhoY0 = rhoY0; ex.strat_inv = strat_inv; ex.pw = pw;
    return ex;
}

}  // namespace

extern "C" {

void adv_host_mass(const int *geo, const double *dg, double **fields, double **faces) {
    HostEx ex = make(geo, dg, 0, fields, faces, nullptr, nullptr, nullptr);
    ex.mass();
}

void adv_host_strang(const int *geo, const double *dg, int comp, double **fields, double **faces,
                     const double *rhoY0, const double *strat_inv, double dt, int odd) {
    HostEx ex = make(geo, dg, comp, fields, faces, rhoY0, strat_inv, nullptr);
    adv_strang(ex, ex.G, dt, odd);
}

void adv_host_rk(const int *geo, const double *dg, int comp, double **fields, double **faces,
                 const double *rhoY0, const double *strat_inv, double dt, double *pwchi) {
    HostEx ex = make(geo, dg, comp, fields, faces, rhoY0, strat_inv, pwchi);
    adv_rk(ex, ex.G, dt);
}

}
