// transport_host.cpp -- the device bodies of the CLSVOF transport
// (simcoflow3d_gb300/csrc/transport_body.cuh), compiled for the host with
// every index range-checked, driven over the same thread indices as the
// kernels of k_transport.cu, one after the other.  Test infrastructure: it
// lets the CPU tests check the kernels' index arithmetic and arithmetic
// against the oracle without a GPU.
#define TR_HOST_CHECK 1
#include <string.h>

#include <vector>

#include "transport_body.cuh"

using tr::Dims;
using tr::Geo;

extern "C" int host_clsvof_step(int I, int J, int K, const double *const geo[6], double *vofl, double *phil,
                                double *nxl, double *nyl, double *nzl, const double *const fn[3],
                                const double *const vel[3], const double *const bc_vel[3], double *const lvs_bc[6],
                                double *const vof_bc[6], const int lvs_flag[6], const double lvs_const[6],
                                const int vof_flag[6], const double vof_const[6], double dt)
{
    const Dims D{I, J, K};
    const Geo G{geo[0], geo[1], geo[2], geo[3], geo[4], geo[5]};
    const size_t nin = D.interior(), ng = D.ghosted();
    std::vector<double> vf[3], ls[3], nx(ng), ny(ng), nz(ng), dis(ng);
    for (int b = 0; b < 3; ++b) {
        vf[b].assign(ng, 0.0);
        ls[b].assign(ng, 0.0);
    }
    std::vector<unsigned long long> key(nin);
    std::vector<uint8_t> fix(nin);
    for (int b = 0; b < 3; ++b) {   // staging fills all three buffers
        memcpy(vf[b].data(), vofl, ng * sizeof(double));
        memcpy(ls[b].data(), phil, ng * sizeof(double));
    }
    const double dtv = dt / (double)tr::NSUB;
    auto cells = [&](auto &&body) {   // the 3-D grid of the interior kernels
        for (int k = 1; k <= K; ++k)
            for (int j = 1; j <= J; ++j)
                for (int i = 1; i <= I; ++i) body(i, j, k);
    };
    auto reconstruct = [&](int cur, bool tail) {
        cells([&](int i, int j, int k) {   // k_reconstruct
            double n1, n2, n3, d1;
            tr::reconstruct(D, G, vf[cur].data(), ls[cur].data(), i, j, k, n1, n2, n3, d1);
            const size_t g = D.g(i, j, k), t = D.n(i, j, k);
            nx[g] = n1;
            ny[g] = n2;
            nz[g] = n3;
            if (tail) {
                nxl[g] = n1;
                nyl[g] = n2;
                nzl[g] = n3;
                d1 = (0.5 * G.dx[t] * fabs(n1) + 0.5 * G.dy[t] * fabs(n2) + 0.5 * G.dz[t] * fabs(n3)) - d1;
            }
            dis[g] = d1;
        });
    };
    for (int kk = 1; kk <= tr::NSUB; ++kk) {
        const int first = kk % 3 == 0 ? 0 : kk % 3 == 1 ? 1 : 2;
        int cur = 0;
        for (int s = 0; s < 3; ++s) {
            const int ax = (first + s) % 3, out = s == 0 ? 1 : s == 1 ? 2 : 0;
            reconstruct(cur, false);
            tr::SweepIn S;
            S.vfl = vf[cur].data();
            S.phi = ls[cur].data();
            S.nx = nx.data();
            S.ny = ny.data();
            S.nz = nz.data();
            S.dis = dis.data();
            S.vel = vel[ax];
            S.bc_vel = bc_vel[ax];
            S.bc_lvs = lvs_bc[2 * ax];
            S.vf_first = vf[1].data();
            S.ls_first = ls[1].data();
            S.dtv = dtv;
            S.axis = ax;
            S.stage = s;
            cells([&](int i, int j, int k) {   // k_sweep: interior only
                double a, b;
                tr::sweep_cell(D, G, S, i, j, k, a, b);
                const size_t t = D.g(i, j, k);
                vf[out][t] = a;
                ls[out][t] = b;
            });
            cur = out;
        }
        tr::WallIn W;
        W.phil = ls[0].data();
        W.vofl = vf[0].data();
        for (int q = 0; q < 2; ++q) {   // k_walls keeps the buffers' ghosts alike
            W.phil_more[q] = ls[q + 1].data();
            W.vofl_more[q] = vf[q + 1].data();
        }
        W.nxl = nxl;
        W.nx = fn[0];
        W.ny = fn[1];
        W.nz = fn[2];
        for (int f = 0; f < 6; ++f) {
            W.lvs_bc[f] = lvs_bc[f];
            W.vof_bc[f] = vof_bc[f];
            W.lvs_flag[f] = lvs_flag[f];
            W.vof_flag[f] = vof_flag[f];
            W.lvs_const[f] = lvs_const[f];
            W.vof_const[f] = vof_const[f];
        }
        for (int axis = 0; axis < 3; ++axis)   // k_walls
            for (size_t t = 0; t < D.plane_size(axis); ++t) tr::wall_point(D, G, W, axis, t);
        reconstruct(0, true);
        std::vector<uint32_t> list;
        cells([&](int i, int j, int k) {   // k_band_reset: reset, list the interface cells
            const size_t c = D.n(i, j, k);
            key[c] = (unsigned long long)tr::key_of(1.0e4);
            fix[c] = 0;
            if (tr::band_interface(vf[0][D.g(i, j, k)])) list.push_back((uint32_t)c);
        });
        for (size_t q = list.size(); q-- > 0;) {   // k_band_pairs (any order of cells and pairs)
            int i, j, k;
            tr::cell_of(D, list[q], i, j, k);
            TR_CHECK(D.n(i, j, k) == list[q], "cell_of");
            for (int t = tr::BAND_CELLS; t-- > 0;)
                tr::band_pair(D, G, vf[0].data(), ls[0].data(), nx.data(), ny.data(), nz.data(), dis.data(), i, j, k,
                              t, key.data(), fix.data());
        }
        cells([&](int i, int j, int k) {   // k_band_value
            ls[0][D.g(i, j, k)] = tr::band_value(D, G, vf[0].data(), dis.data(), i, j, k, key.data(), fix.data());
        });
    }
    memcpy(vofl, vf[0].data(), ng * sizeof(double));
    memcpy(phil, ls[0].data(), ng * sizeof(double));
    return 0;
}

// ComputeUVWLiquidField: k_uvw for the three families over the ghosted grid.
// pd: the P spacings (interior); pf: the P cells' phiL, nxL, nyL, nzL, vofL;
// vg[f]: family f's spacings; vf[f]: its phiL, nxL, nyL, nzL, vofL (in/out).
extern "C" int host_uvw(int I, int J, int K, const double *const pd[3], const double *const pf[5],
                        const double *const vg[9], double *const vf[15])
{
    const Dims D{I, J, K};
    const Geo G{nullptr, nullptr, nullptr, pd[0], pd[1], pd[2]};
    const double *pin[4] = {pf[0], pf[1], pf[2], pf[3]};
    for (int fam = 0; fam < 3; ++fam) {
        const double *d = fam == 0 ? G.dx : fam == 1 ? G.dy : G.dz;
        double *const *o = vf + 5 * fam;
        for (int k = 0; k <= K + 1; ++k)   // k_uvw's 3-D grid over the ghosted cells
            for (int j = 0; j <= J + 1; ++j)
                for (int i = 0; i <= I + 1; ++i) {
                    const size_t t = D.g(i, j, k);
                    if (i < I && j < J && k < K) {
                        double av[4];
                        tr::family_average(D, fam, d, pin, i, j, k, av);
                        for (int q = 0; q < 4; ++q) o[q][t] = av[q];
                    }
                    if (i >= 1 && i <= I && j >= 1 && j <= J && k >= 1 && k <= K)
                        o[4][t] = tr::family_vofl(D, fam, G.dx, G.dy, G.dz, pf[0], pf[1], pf[2], pf[3], pf[4],
                                                  vg[3 * fam], vg[3 * fam + 1], vg[3 * fam + 2], i, j, k);
                }
    }
    return 0;
}
