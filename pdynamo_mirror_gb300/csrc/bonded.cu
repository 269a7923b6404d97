// bonded.cu - harmonic bond and angle terms of an MM model (pdg_mm_bonded_*, include/pdg.h), for many frames.
//
// E_bond  = k (r - r0)^2                       (HarmonicBondContainer_Energy, pMolecule-1.9.0/extensions/csource/
//                                               HarmonicBondContainer.c:149-181)
// E_angle = k (theta - theta0)^2, theta at j   (HarmonicAngleContainer_Energy, HarmonicAngleContainer.c:157-200; the
//                                               cosine clamped to +-0.999999 as the reference's DOT_LIMIT)
// Energies in kJ/mol, coordinates in Angstrom, gradients in kJ/mol/A.  Two kernels, no scratch: the energies of a frame
// are summed by one block in a fixed order; the gradient of an atom by one thread that recomputes each of its terms from
// a per-atom term list (term index and the atom's role in it), so every gradient is its own fixed-order sum.
#include "common.cuh"

#define BT 256

struct BondedDevice {
    int n_atoms, n_bonds, n_angles;
    const int *bonds;          // 2 per bond
    const double *bond_p;      // r0, k per bond
    const int *angles;         // i, j (apex), k per angle
    const double *angle_p;     // theta0 (rad), k per angle
    const int *bstart, *blist; // per atom: bond entries (bond * 2 + role)
    const int *astart, *alist; // per atom: angle entries (angle * 4 + role)
};

__device__ __forceinline__ double bond_term(const double *x, const BondedDevice &b, int t, double g[3], int role)
{
    const int i = b.bonds[2 * t], j = b.bonds[2 * t + 1];
    const double xij = x[3 * i] - x[3 * j], yij = x[3 * i + 1] - x[3 * j + 1], zij = x[3 * i + 2] - x[3 * j + 2];
    const double rij = sqrt(xij * xij + yij * yij + zij * zij);
    const double disp = rij - b.bond_p[2 * t], df = b.bond_p[2 * t + 1] * disp;
    if (g) {
        const double s = (role == 0 ? 2.0 : -2.0) * df / rij;
        g[0] += s * xij; g[1] += s * yij; g[2] += s * zij;
    }
    return df * disp;
}

__device__ __forceinline__ double angle_term(const double *x, const BondedDevice &b, int t, double g[3], int role)
{
    const int i = b.angles[3 * t], j = b.angles[3 * t + 1], k = b.angles[3 * t + 2];
    double xij = x[3 * i] - x[3 * j], yij = x[3 * i + 1] - x[3 * j + 1], zij = x[3 * i + 2] - x[3 * j + 2];
    double xkj = x[3 * k] - x[3 * j], ykj = x[3 * k + 1] - x[3 * j + 1], zkj = x[3 * k + 2] - x[3 * j + 2];
    const double rij = sqrt(xij * xij + yij * yij + zij * zij), rkj = sqrt(xkj * xkj + ykj * ykj + zkj * zkj);
    xij /= rij; yij /= rij; zij /= rij; xkj /= rkj; ykj /= rkj; zkj /= rkj;
    double dot = xij * xkj + yij * ykj + zij * zkj;
    dot = fmin(0.999999, fmax(-0.999999, dot));
    const double theta = acos(dot), disp = theta - b.angle_p[2 * t], df = b.angle_p[2 * t + 1] * disp;
    if (g) {
        const double d2 = df * 2.0 * (-1.0 / sqrt(1.0 - dot * dot));
        const double ti[3] = { d2 * (xkj - dot * xij) / rij, d2 * (ykj - dot * yij) / rij, d2 * (zkj - dot * zij) / rij };
        const double tk[3] = { d2 * (xij - dot * xkj) / rkj, d2 * (yij - dot * ykj) / rkj, d2 * (zij - dot * zkj) / rkj };
        for (int c = 0; c < 3; c++) g[c] += role == 0 ? ti[c] : (role == 2 ? tk[c] : -(ti[c] + tk[c]));
    }
    return df * disp;
}

__global__ void __launch_bounds__(BT) k_bonded_energies(BondedDevice b, const double *__restrict__ xyz, double *__restrict__ energies)
{
    __shared__ double red[32];
    const int f = blockIdx.x;
    const double *x = xyz + (size_t)f * b.n_atoms * 3;
    double eb = 0.0, ea = 0.0;
    for (int t = threadIdx.x; t < b.n_bonds; t += BT) eb += bond_term(x, b, t, nullptr, 0);
    for (int t = threadIdx.x; t < b.n_angles; t += BT) ea += angle_term(x, b, t, nullptr, 0);
    eb = block_sum(eb, red);
    ea = block_sum(ea, red);
    if (threadIdx.x == 0) { energies[2 * f] = eb; energies[2 * f + 1] = ea; }
}

__global__ void __launch_bounds__(BT) k_bonded_gradients(BondedDevice b, int n_frames, const double *__restrict__ xyz, double *__restrict__ grad)
{
    const long g = (long)blockIdx.x * BT + threadIdx.x;
    if (g >= (long)n_frames * b.n_atoms) return;
    const int f = (int)(g / b.n_atoms), a = (int)(g % b.n_atoms);
    const int b0 = b.bstart[a], b1 = b.bstart[a + 1], a0 = b.astart[a], a1 = b.astart[a + 1];
    if (b0 == b1 && a0 == a1) return;
    const double *x = xyz + (size_t)f * b.n_atoms * 3;
    double acc[3] = { 0.0, 0.0, 0.0 };
    for (int e = b0; e < b1; e++) bond_term(x, b, b.blist[e] >> 1, acc, b.blist[e] & 1);
    for (int e = a0; e < a1; e++) angle_term(x, b, b.alist[e] >> 2, acc, b.alist[e] & 3);
    double *o = grad + ((size_t)f * b.n_atoms + a) * 3;
    o[0] += acc[0]; o[1] += acc[1]; o[2] += acc[2];
}

void launch_bonded(const BondedDevice &b, int n_frames, const double *xyz, double *energies, double *grad, cudaStream_t st)
{
    if (energies) k_bonded_energies<<<n_frames, BT, 0, st>>>(b, xyz, energies);
    if (grad) {
        const long n = (long)n_frames * b.n_atoms;
        k_bonded_gradients<<<(unsigned)((n + BT - 1) / BT), BT, 0, st>>>(b, n_frames, xyz, grad);
    }
}

// ---------------------------------------------------------------------------------------------------------------
// Host side: the C ABI.
#include <vector>
#include <string>

struct pdg_mm_bonded {
    BondedDevice d;
    void *mem = nullptr;
};

int bonded_fail(int code, const char *msg);   // api.cu: records the message for pdg_last_error

extern "C" int pdg_mm_bonded_create(int n_atoms, int n_bonds, const int *h_bonds, const double *h_bond_params, int n_angles,
                                    const int *h_angles, const double *h_angle_params, pdg_mm_bonded **out)
{
    if (!out || n_atoms <= 0 || n_bonds < 0 || n_angles < 0 || (n_bonds > 0 && (!h_bonds || !h_bond_params)) ||
        (n_angles > 0 && (!h_angles || !h_angle_params)))
        return bonded_fail(PDG_BAD_ARGUMENT, "pdg_mm_bonded_create: bad argument");
    for (int t = 0; t < 2 * n_bonds; t++)
        if (h_bonds[t] < 0 || h_bonds[t] >= n_atoms) return bonded_fail(PDG_BAD_ARGUMENT, "pdg_mm_bonded_create: bond atom out of range");
    for (int t = 0; t < 3 * n_angles; t++)
        if (h_angles[t] < 0 || h_angles[t] >= n_atoms) return bonded_fail(PDG_BAD_ARGUMENT, "pdg_mm_bonded_create: angle atom out of range");
    for (int t = 0; t < n_bonds; t++)
        if (h_bonds[2 * t] == h_bonds[2 * t + 1]) return bonded_fail(PDG_BAD_ARGUMENT, "pdg_mm_bonded_create: a bond joins an atom to itself");
    for (int t = 0; t < n_angles; t++) {
        const int *q = h_angles + 3 * t;
        if (q[0] == q[1] || q[1] == q[2] || q[0] == q[2]) return bonded_fail(PDG_BAD_ARGUMENT, "pdg_mm_bonded_create: an angle repeats an atom");
    }
    // per-atom term lists, terms in increasing order
    std::vector<int> bstart(n_atoms + 1, 0), astart(n_atoms + 1, 0);
    for (int t = 0; t < n_bonds; t++) for (int r = 0; r < 2; r++) bstart[h_bonds[2 * t + r] + 1]++;
    for (int t = 0; t < n_angles; t++) for (int r = 0; r < 3; r++) astart[h_angles[3 * t + r] + 1]++;
    for (int a = 0; a < n_atoms; a++) { bstart[a + 1] += bstart[a]; astart[a + 1] += astart[a]; }
    std::vector<int> blist(2 * (size_t)n_bonds), alist(3 * (size_t)n_angles), bf(bstart.begin(), bstart.end() - 1), af(astart.begin(), astart.end() - 1);
    for (int t = 0; t < n_bonds; t++) for (int r = 0; r < 2; r++) blist[bf[h_bonds[2 * t + r]]++] = t * 2 + r;
    for (int t = 0; t < n_angles; t++) for (int r = 0; r < 3; r++) alist[af[h_angles[3 * t + r]]++] = t * 4 + r;
    // one allocation: doubles first, then ints
    const size_t nd = 2 * (size_t)n_bonds + 2 * (size_t)n_angles;
    const size_t ni = 2 * (size_t)n_bonds + 3 * (size_t)n_angles + 2 * (size_t)(n_atoms + 1) + blist.size() + alist.size();
    pdg_mm_bonded *B = new pdg_mm_bonded();
    if (cudaMalloc(&B->mem, sizeof(double) * nd + sizeof(int) * ni + 16) != cudaSuccess) { delete B; return bonded_fail(PDG_CUDA_ERROR, "pdg_mm_bonded_create: device allocation failed"); }
    double *dd = (double *)B->mem;
    int *di = (int *)(dd + nd);
    std::vector<double> hd(nd);
    std::vector<int> hi;
    hi.reserve(ni);
    for (size_t k = 0; k < 2 * (size_t)n_bonds; k++) hd[k] = h_bond_params[k];
    for (size_t k = 0; k < 2 * (size_t)n_angles; k++) hd[2 * (size_t)n_bonds + k] = h_angle_params[k];
    hi.insert(hi.end(), h_bonds, h_bonds + 2 * (size_t)n_bonds);
    hi.insert(hi.end(), h_angles, h_angles + 3 * (size_t)n_angles);
    hi.insert(hi.end(), bstart.begin(), bstart.end());
    hi.insert(hi.end(), astart.begin(), astart.end());
    hi.insert(hi.end(), blist.begin(), blist.end());
    hi.insert(hi.end(), alist.begin(), alist.end());
    if (cudaMemcpy(dd, hd.data(), sizeof(double) * nd, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(di, hi.data(), sizeof(int) * ni, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(B->mem); delete B;
        return bonded_fail(PDG_CUDA_ERROR, "pdg_mm_bonded_create: copy to the device failed");
    }
    BondedDevice &d = B->d;
    d.n_atoms = n_atoms; d.n_bonds = n_bonds; d.n_angles = n_angles;
    d.bond_p = dd; d.angle_p = dd + 2 * (size_t)n_bonds;
    d.bonds = di; d.angles = di + 2 * (size_t)n_bonds;
    d.bstart = d.angles + 3 * (size_t)n_angles; d.astart = d.bstart + n_atoms + 1;
    d.blist = d.astart + n_atoms + 1; d.alist = d.blist + blist.size();
    *out = B;
    return PDG_OK;
}

extern "C" int pdg_mm_bonded_destroy(pdg_mm_bonded *b)
{
    if (!b) return PDG_OK;
    if (b->mem) cudaFree(b->mem);
    delete b;
    return PDG_OK;
}

extern "C" int pdg_mm_bonded_energy_gradients(const pdg_mm_bonded *b, int n_frames, const double *d_xyz, double *d_energies,
                                              double *d_gradients, void *stream)
{
    if (!b || n_frames <= 0 || n_frames > 65535 || !d_xyz || (!d_energies && !d_gradients))
        return bonded_fail(PDG_BAD_ARGUMENT, "pdg_mm_bonded_energy_gradients: bad argument");
    launch_bonded(b->d, n_frames, d_xyz, d_energies, d_gradients, (cudaStream_t)stream);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PDG_OK : bonded_fail(PDG_CUDA_ERROR, "pdg_mm_bonded_energy_gradients: kernel launch failed");
}
