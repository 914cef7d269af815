#include "problems.h"

#include <algorithm>
#include <cmath>

#include "rng.h"

namespace rschol {

namespace {

void draw_rhs(MT19937& gen, Problem& P, int nrhs, bool uniform) {
  P.nrhs = nrhs;
  P.rhs.assign((size_t)P.n * nrhs, 0.0);
  for (size_t i = 0; i < P.rhs.size(); ++i)
    P.rhs[i] = uniform ? (-1.0 + 2.0 * gen.randExc()) : gen.randNorm(0.0, 1.0);
}

}  // namespace

Problem make_diffusion(int dim, int nx, int ny, int nz, double sigma,
                       uint32_t seed, int nrhs) {
  if (dim == 2) nz = 1;
  Problem P;
  const int n = nx * ny * nz;
  P.n = n;
  MT19937 gen(seed);
  std::vector<double> kappa(n, 1.0);
  if (sigma != 0.0)
    for (int i = 0; i < n; ++i) kappa[i] = std::exp(sigma * gen.randNorm(0.0, 1.0));

  auto id = [&](int i, int j, int k) { return i + nx * (j + ny * k); };
  auto face = [&](int a, int b) { return 2.0 * kappa[a] * kappa[b] / (kappa[a] + kappa[b]); };

  P.colptr.assign(n + 1, 0);
  P.rowind.reserve((size_t)n * (2 * dim + 1));
  P.vals.reserve((size_t)n * (2 * dim + 1));
  P.xyz.resize(3 * (size_t)n);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int c = id(i, j, k);
        P.xyz[3 * (size_t)c + 0] = i;
        P.xyz[3 * (size_t)c + 1] = j;
        P.xyz[3 * (size_t)c + 2] = k;
        // neighbours in increasing index order: -z, -y, -x, self, +x, +y, +z
        double diag = 0.0;
        struct E { int r; double v; } ent[7];
        int ne = 0;
        const int di[6] = {0, 0, -1, 1, 0, 0};
        const int dj[6] = {0, -1, 0, 0, 1, 0};
        const int dk[6] = {-1, 0, 0, 0, 0, 1};
        for (int f = 0; f < 6; ++f) {
          if (dim == 2 && dk[f] != 0) continue;
          int ii = i + di[f], jj = j + dj[f], kk = k + dk[f];
          bool inside = ii >= 0 && ii < nx && jj >= 0 && jj < ny && kk >= 0 && kk < nz;
          if (inside) {
            double t = face(c, id(ii, jj, kk));
            diag += t;
            ent[ne++] = {id(ii, jj, kk), -t};
          } else {
            diag += kappa[c];
          }
          if (f == 2) ent[ne++] = {c, 0.0};  // diagonal slot after -x
        }
        for (int e = 0; e < ne; ++e) {
          if (ent[e].r == c) ent[e].v = diag;
          P.rowind.push_back(ent[e].r);
          P.vals.push_back(ent[e].v);
        }
        P.colptr[c + 1] = (int)P.rowind.size();
      }
  draw_rhs(gen, P, nrhs, false);
  return P;
}

Problem make_elasticity(int ne, double E, double nu, uint32_t seed, int nrhs) {
  const int nn1 = ne + 1;
  const int nnodes = nn1 * nn1 * nn1;
  const double h = 1.0 / ne;
  const double lam = E * nu / ((1 + nu) * (1 - 2 * nu));
  const double mu = E / (2 * (1 + nu));

  // Element stiffness (24 x 24), identical for every element of the mesh.
  double Ke[24][24] = {};
  const double g = 1.0 / std::sqrt(3.0);
  const double detJ = (h / 2) * (h / 2) * (h / 2);
  for (int gz = 0; gz < 2; ++gz)
    for (int gy = 0; gy < 2; ++gy)
      for (int gx = 0; gx < 2; ++gx) {
        double xi = gx ? g : -g, eta = gy ? g : -g, zeta = gz ? g : -g;
        double dN[8][3];
        for (int a = 0; a < 8; ++a) {
          double xa = (a & 1) ? 1 : -1, ya = (a & 2) ? 1 : -1, za = (a & 4) ? 1 : -1;
          dN[a][0] = xa * (1 + eta * ya) * (1 + zeta * za) / 8 * (2 / h);
          dN[a][1] = ya * (1 + xi * xa) * (1 + zeta * za) / 8 * (2 / h);
          dN[a][2] = za * (1 + xi * xa) * (1 + eta * ya) / 8 * (2 / h);
        }
        double B[6][24] = {};
        for (int a = 0; a < 8; ++a) {
          B[0][3 * a + 0] = dN[a][0];
          B[1][3 * a + 1] = dN[a][1];
          B[2][3 * a + 2] = dN[a][2];
          B[3][3 * a + 0] = dN[a][1]; B[3][3 * a + 1] = dN[a][0];
          B[4][3 * a + 1] = dN[a][2]; B[4][3 * a + 2] = dN[a][1];
          B[5][3 * a + 0] = dN[a][2]; B[5][3 * a + 2] = dN[a][0];
        }
        double D[6][6] = {};
        for (int r = 0; r < 3; ++r)
          for (int s = 0; s < 3; ++s) D[r][s] = lam + (r == s ? 2 * mu : 0.0);
        D[3][3] = D[4][4] = D[5][5] = mu;
        double DB[6][24];
        for (int r = 0; r < 6; ++r)
          for (int c = 0; c < 24; ++c) {
            double s = 0;
            for (int t = 0; t < 6; ++t) s += D[r][t] * B[t][c];
            DB[r][c] = s;
          }
        for (int r = 0; r < 24; ++r)
          for (int c = 0; c < 24; ++c) {
            double s = 0;
            for (int t = 0; t < 6; ++t) s += B[t][r] * DB[t][c];
            Ke[r][c] += s * detJ;
          }
      }

  // Node-level 27-point structure: pos[node*27 + o] = slot of neighbour o.
  auto nid = [&](int x, int y, int z) { return x + nn1 * (y + nn1 * z); };
  std::vector<int> nbrStart(nnodes + 1, 0), pos((size_t)nnodes * 27, -1);
  for (int z = 0; z < nn1; ++z)
    for (int y = 0; y < nn1; ++y)
      for (int x = 0; x < nn1; ++x) {
        int p = nid(x, y, z), cnt = 0;
        for (int o = 0; o < 27; ++o) {
          int dx = o % 3 - 1, dy = (o / 3) % 3 - 1, dz = o / 9 - 1;
          int qx = x + dx, qy = y + dy, qz = z + dz;
          if (qx < 0 || qy < 0 || qz < 0 || qx >= nn1 || qy >= nn1 || qz >= nn1) continue;
          pos[(size_t)p * 27 + o] = cnt++;
        }
        nbrStart[p + 1] = nbrStart[p] + cnt;
      }
  // Full (all-dof) block values: 9 doubles per node-neighbour slot.
  std::vector<double> blk((size_t)nbrStart[nnodes] * 9, 0.0);
  for (int ez = 0; ez < ne; ++ez)
    for (int ey = 0; ey < ne; ++ey)
      for (int ex = 0; ex < ne; ++ex)
        for (int a = 0; a < 8; ++a) {
          int ax = ex + (a & 1), ay = ey + ((a >> 1) & 1), az = ez + ((a >> 2) & 1);
          int pa = nid(ax, ay, az);
          for (int b = 0; b < 8; ++b) {
            int bx = ex + (b & 1), by = ey + ((b >> 1) & 1), bz = ez + ((b >> 2) & 1);
            int o = (bx - ax + 1) + 3 * (by - ay + 1) + 9 * (bz - az + 1);
            double* dst = &blk[((size_t)nbrStart[pa] + pos[(size_t)pa * 27 + o]) * 9];
            for (int da = 0; da < 3; ++da)
              for (int db = 0; db < 3; ++db) dst[da * 3 + db] += Ke[3 * a + da][3 * b + db];
          }
        }

  // Free dofs: nodes with x > 0 (the x = 0 face is clamped and eliminated).
  std::vector<int> dofOf((size_t)nnodes * 3, -1);
  int n = 0;
  for (int p = 0; p < nnodes; ++p) {
    int x = p % nn1;
    if (x == 0) continue;
    for (int d = 0; d < 3; ++d) dofOf[(size_t)p * 3 + d] = n++;
  }
  Problem P;
  P.n = n;
  P.colptr.assign(n + 1, 0);
  P.rowind.reserve((size_t)n * 81);
  P.vals.reserve((size_t)n * 81);
  P.xyz.resize(3 * (size_t)n);
  for (int p = 0; p < nnodes; ++p) {
    int x = p % nn1, y = (p / nn1) % nn1, z = p / (nn1 * nn1);
    if (x == 0) continue;
    for (int da = 0; da < 3; ++da) {
      int row = dofOf[(size_t)p * 3 + da];
      P.xyz[3 * (size_t)row + 0] = x * h;
      P.xyz[3 * (size_t)row + 1] = y * h;
      P.xyz[3 * (size_t)row + 2] = z * h;
      for (int o = 0; o < 27; ++o) {
        int slot = pos[(size_t)p * 27 + o];
        if (slot < 0) continue;
        int dx = o % 3 - 1, dy = (o / 3) % 3 - 1, dz = o / 9 - 1;
        int q = nid(x + dx, y + dy, z + dz);
        if (q % nn1 == 0) continue;
        const double* src = &blk[((size_t)nbrStart[p] + slot) * 9];
        for (int db = 0; db < 3; ++db) {
          P.rowind.push_back(dofOf[(size_t)q * 3 + db]);
          P.vals.push_back(src[da * 3 + db]);
        }
      }
      P.colptr[row + 1] = (int)P.rowind.size();
    }
  }
  MT19937 gen(seed);
  draw_rhs(gen, P, nrhs, true);
  return P;
}

}  // namespace rschol
