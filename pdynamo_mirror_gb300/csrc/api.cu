// api.cu - the extern "C" boundary of libpdg.so (declared in include/pdg.h).
#include <cstdio>
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "multipole.cuh"
#include "overlap.cuh"

static thread_local std::string g_error;

static int fail(int code, const std::string &msg)
{
    g_error = msg;
    return code;
}

static int cuda_check(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) return fail(PDG_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
    return PDG_OK;
}

struct pdg_system {
    DeviceSystem d;
    std::vector<double> elements;
    int charge;
    // device allocations owned by the system (tables only; no per-frame data)
    double *d_elements = nullptr, *d_terms = nullptr, *d_ovl = nullptr, *d_ovl_tab = nullptr;
    int *d_ovl_tab_idx = nullptr;   // per ordered element pair: table offset, then node count
    float *d_ovl32 = nullptr, *d_mpw32 = nullptr;
    int *d_ints = nullptr;
    void *d_mp = nullptr;
    // phase events of pdg_energy_gradients (pdg_phase_events / pdg_phase_times): before the integrals, after them,
    // after the SCF, after the gradients
    cudaEvent_t ev[4] = { nullptr, nullptr, nullptr, nullptr };
    int ev_on = 0, ev_recorded = 0;
    // shared base of the mixed method's perturbative density steps (caller-owned device memory, pdg_set_shared_base)
    const double *shared_base = nullptr;
    // side stream of pdg_set_side_stream and the two events that order it against the SCF
    cudaStream_t side = nullptr;
    cudaEvent_t side_in = nullptr, scf_out = nullptr;
};

extern "C" int pdg_version(void) { return 100; }

int bonded_fail(int code, const char *msg) { return fail(code, msg); }

extern "C" const char *pdg_last_error(void) { return g_error.c_str(); }

extern "C" int pdg_system_create(const double *h_elements, int n_elements, int n_atoms, const int *h_atom_element,
                                 int charge, pdg_system **out)
{
    if (!out || !h_elements || !h_atom_element) return fail(PDG_BAD_ARGUMENT, "null argument");
    *out = nullptr;
    if (n_elements <= 0 || n_elements > PDG_MAX_ELEMENTS) return fail(PDG_TOO_LARGE, "element count outside 1..16");
    if (n_atoms <= 0 || n_atoms > PDG_MAX_ATOMS) return fail(PDG_TOO_LARGE, "atom count outside 1..1024");
    for (int e = 0; e < n_elements; e++)   // PM6 records index their diatomic pairs by the partner's place in this list
        if (h_elements[e * PDG_ELEMENT_STRIDE + PDG_E_DIAT] != 0.0 && (int)h_elements[e * PDG_ELEMENT_STRIDE + PDG_E_INDEX] != e)
            return fail(PDG_BAD_ARGUMENT, "PM6 element record whose index is not its place in the element list");
    std::vector<int> elem(n_atoms), start(n_atoms), norb(n_atoms);
    int nb = 0, zsum = 0;
    for (int a = 0; a < n_atoms; a++) {
        int e = h_atom_element[a];
        if (e < 0 || e >= n_elements) return fail(PDG_BAD_ARGUMENT, "atom element index out of range");
        int no = (int)h_elements[e * PDG_ELEMENT_STRIDE + PDG_E_NORB];
        if (no != 1 && no != 4) return fail(PDG_BAD_ARGUMENT, "only s and sp elements are supported");
        elem[a] = e; start[a] = nb; norb[a] = no; nb += no;
        zsum += (int)llround(h_elements[e * PDG_ELEMENT_STRIDE + PDG_E_ZCORE]);
    }
    if (nb > PDG_MAX_BASIS) return fail(PDG_TOO_LARGE, "more than 2048 basis functions");
    int nel = zsum - charge;
    if (nel < 0 || nel > 2 * nb) return fail(PDG_BAD_ARGUMENT, "the electron count does not fit the basis");
    int npairs = n_atoms * (n_atoms - 1) / 2;
    std::vector<int> pi(npairs), pj(npairs), pt(npairs);
    int tei = 0;
    for (int i = 0, p = 0; i < n_atoms; i++)
        for (int j = 0; j < i; j++, p++) {
            pi[p] = i; pj[p] = j; pt[p] = tei;
            tei += (norb[i] * (norb[i] + 1) / 2) * (norb[j] * (norb[j] + 1) / 2);
        }
    // multipole term tables per ordered element pair
    std::vector<double> terms((size_t)n_elements * n_elements * 2 * MP_NTERMS);
    for (int a = 0; a < n_elements; a++)
        for (int b = 0; b < n_elements; b++) {
            double *o = &terms[(size_t)(a * n_elements + b) * 2 * MP_NTERMS];
            multipole_terms(h_elements + a * PDG_ELEMENT_STRIDE, h_elements + b * PDG_ELEMENT_STRIDE, o, o + MP_NTERMS);
        }
    // overlap primitive records per ordered element pair
    std::vector<double> ovl;
    std::vector<int> ovl_off(n_elements * n_elements), ovl_n(n_elements * n_elements);
    for (int a = 0; a < n_elements; a++)
        for (int b = 0; b < n_elements; b++) {
            const size_t before = ovl.size() / OV_REC;
            overlap_records(h_elements + a * PDG_ELEMENT_STRIDE, h_elements + b * PDG_ELEMENT_STRIDE, ovl);
            ovl_off[a * n_elements + b] = (int)before;
            ovl_n[a * n_elements + b] = (int)(ovl.size() / OV_REC - before);
        }
    if (ovl.empty()) ovl.assign(OV_REC, 0.0);
    // the same sums tabulated against R (the mixed method's integrals)
    std::vector<double> ovl_tab;
    std::vector<int> ovl_tab_idx(2 * n_elements * n_elements);
    for (int e = 0; e < n_elements * n_elements; e++) {
        ovl_tab_idx[e] = (int)ovl_tab.size();
        ovl_tab_idx[n_elements * n_elements + e] = overlap_table(ovl.data() + (size_t)ovl_off[e] * OV_REC, ovl_n[e], ovl_tab);
    }
    pdg_system *s = new pdg_system();
    s->elements.assign(h_elements, h_elements + (size_t)n_elements * PDG_ELEMENT_STRIDE);
    s->charge = charge;
    std::vector<int> ints;
    ints.insert(ints.end(), elem.begin(), elem.end());
    ints.insert(ints.end(), start.begin(), start.end());
    ints.insert(ints.end(), norb.begin(), norb.end());
    ints.insert(ints.end(), pi.begin(), pi.end());
    ints.insert(ints.end(), pj.begin(), pj.end());
    ints.insert(ints.end(), pt.begin(), pt.end());
    ints.insert(ints.end(), ovl_off.begin(), ovl_off.end());
    ints.insert(ints.end(), ovl_n.begin(), ovl_n.end());
    // Fock output lists: diagonal-block elements per atom; off-diagonal-block elements sorted by pair class
    std::vector<int> cel, xel;
    for (int a = 0; a < n_atoms; a++)
        for (int ab = 0; ab < norb[a] * (norb[a] + 1) / 2; ab++) cel.push_back(a << 4 | ab);
    for (int cls = 16; cls >= 1; cls--)
        for (int p = 0; p < npairs; p++)
            if (norb[pi[p]] * norb[pj[p]] == cls)
                for (int k = 0; k < cls; k++) xel.push_back(p << 4 | k);
    const size_t cel_at = ints.size();
    ints.insert(ints.end(), cel.begin(), cel.end());
    ints.insert(ints.end(), xel.begin(), xel.end());
    // s-s and sp-s pairs (thread-per-pair kernels) and sp-sp pairs (warp-per-pair kernels)
    std::vector<int> pss, pgen, psps;
    for (int p = 0; p < npairs; p++) {
        const int ns = (norb[pi[p]] == 1) + (norb[pj[p]] == 1);
        (ns == 2 ? pss : ns == 1 ? psps : pgen).push_back(p);
    }
    const size_t pl_at = ints.size();
    ints.insert(ints.end(), pss.begin(), pss.end());
    ints.insert(ints.end(), pgen.begin(), pgen.end());
    ints.insert(ints.end(), psps.begin(), psps.end());
    const size_t pk_at = ints.size();
    for (int a = 0, k = 0; a <= n_atoms; a++) { ints.push_back(k); if (a < n_atoms) k += norb[a] * (norb[a] + 1) / 2; }
    MultipoleMap mp;
    if (!multipole_map_spsp(mp)) { pdg_system_destroy(s); return fail(PDG_BAD_ARGUMENT, "multipole map exceeds its term limit"); }
    std::vector<float> ovl32(ovl.begin(), ovl.end()), mpw32(mp.w, mp.w + MP_MAP_MAX * MP_MAP_NNZ);
    int rc = PDG_OK;
    if ((rc = cuda_check(cudaMalloc(&s->d_mp, sizeof(MultipoleMap)), "cudaMalloc multipole map")) ||
        (rc = cuda_check(cudaMemcpy(s->d_mp, &mp, sizeof(MultipoleMap), cudaMemcpyHostToDevice), "copy multipole map")) ||
        (rc = cuda_check(cudaMalloc(&s->d_elements, sizeof(double) * s->elements.size()), "cudaMalloc elements")) ||
        (rc = cuda_check(cudaMalloc(&s->d_terms, sizeof(double) * terms.size()), "cudaMalloc terms")) ||
        (rc = cuda_check(cudaMalloc(&s->d_ints, sizeof(int) * ints.size()), "cudaMalloc tables")) ||
        (rc = cuda_check(cudaMalloc(&s->d_ovl, sizeof(double) * ovl.size()), "cudaMalloc overlap records")) ||
        (rc = cuda_check(cudaMemcpy(s->d_ovl, ovl.data(), sizeof(double) * ovl.size(), cudaMemcpyHostToDevice), "copy overlap records")) ||
        (rc = cuda_check(cudaMalloc(&s->d_ovl32, sizeof(float) * ovl.size()), "cudaMalloc FP32 overlap records")) ||
        (rc = cuda_check(cudaMemcpy(s->d_ovl32, ovl32.data(), sizeof(float) * ovl32.size(), cudaMemcpyHostToDevice), "copy FP32 overlap records")) ||
        (rc = cuda_check(cudaMalloc(&s->d_mpw32, sizeof(float) * MP_MAP_MAX * MP_MAP_NNZ), "cudaMalloc FP32 multipole weights")) ||
        (rc = cuda_check(cudaMemcpy(s->d_mpw32, mpw32.data(), sizeof(float) * mpw32.size(), cudaMemcpyHostToDevice), "copy FP32 multipole weights")) ||
        (rc = cuda_check(cudaMemcpy(s->d_elements, s->elements.data(), sizeof(double) * s->elements.size(), cudaMemcpyHostToDevice), "copy elements")) ||
        (rc = cuda_check(cudaMemcpy(s->d_terms, terms.data(), sizeof(double) * terms.size(), cudaMemcpyHostToDevice), "copy terms")) ||
        (rc = cuda_check(cudaMemcpy(s->d_ints, ints.data(), sizeof(int) * ints.size(), cudaMemcpyHostToDevice), "copy tables")) ||
        (rc = cuda_check(cudaMalloc(&s->d_ovl_tab, sizeof(double) * ovl_tab.size()), "cudaMalloc overlap table")) ||
        (rc = cuda_check(cudaMemcpy(s->d_ovl_tab, ovl_tab.data(), sizeof(double) * ovl_tab.size(), cudaMemcpyHostToDevice), "copy overlap table")) ||
        (rc = cuda_check(cudaMalloc(&s->d_ovl_tab_idx, sizeof(int) * ovl_tab_idx.size()), "cudaMalloc overlap table index")) ||
        (rc = cuda_check(cudaMemcpy(s->d_ovl_tab_idx, ovl_tab_idx.data(), sizeof(int) * ovl_tab_idx.size(), cudaMemcpyHostToDevice),
                         "copy overlap table index"))) {
        pdg_system_destroy(s);
        return rc;
    }
    DeviceSystem &d = s->d;
    d.n_atoms = n_atoms; d.n_basis = nb; d.n_occ = nel / 2; d.n_pairs = npairs; d.n_elements = n_elements;
    d.n_electrons = nel; d.tei_total = tei;
    d.vec_occupied = (d.n_occ <= nb - d.n_occ) ? 1 : 0;
    d.n_vec = d.vec_occupied ? d.n_occ : nb - d.n_occ;
    d.elements = s->d_elements; d.terms = s->d_terms;
    const int *b = s->d_ints;
    d.atom_elem = b; d.atom_start = b + n_atoms; d.atom_norb = b + 2 * n_atoms;
    d.pair_i = b + 3 * n_atoms; d.pair_j = d.pair_i + npairs; d.pair_tei = d.pair_j + npairs;
    d.ovl = s->d_ovl; d.ovl_off = d.pair_tei + npairs; d.ovl_n = d.ovl_off + n_elements * n_elements;
    d.cel = b + cel_at; d.xel = d.cel + cel.size(); d.n_cel = (int)cel.size(); d.n_xel = (int)xel.size();
    d.pairs_ss = b + pl_at; d.pairs_gen = d.pairs_ss + pss.size(); d.n_ss = (int)pss.size(); d.n_gen = (int)pgen.size();
    d.pairs_sps = d.pairs_gen + pgen.size(); d.n_sps = (int)psps.size();
    d.mp_map = s->d_mp;
    d.atom_pk = b + pk_at;
    d.ovl32 = s->d_ovl32; d.mp_w32 = s->d_mpw32;
    d.ovl_tab = nullptr;   // attached per call for the mixed method (mixed_view)
    d.ovl_tab_off = s->d_ovl_tab_idx; d.ovl_tab_n = s->d_ovl_tab_idx + n_elements * n_elements;
    d.ovl_tab_inv_h = 1.0 / OV_TAB_H;
    *out = s;
    return PDG_OK;
}

extern "C" int pdg_system_destroy(pdg_system *s)
{
    if (!s) return PDG_OK;
    cudaFree(s->d_elements); cudaFree(s->d_terms); cudaFree(s->d_ints); cudaFree(s->d_ovl); cudaFree(s->d_mp);
    cudaFree(s->d_ovl32); cudaFree(s->d_mpw32); cudaFree(s->d_ovl_tab); cudaFree(s->d_ovl_tab_idx);
    for (cudaEvent_t e : s->ev)
        if (e) cudaEventDestroy(e);
    if (s->side_in) cudaEventDestroy(s->side_in);
    if (s->scf_out) cudaEventDestroy(s->scf_out);
    delete s;
    return PDG_OK;
}

extern "C" int pdg_system_info(const pdg_system *s, int *n_basis, int *n_occupied, int *n_pairs)
{
    if (!s) return fail(PDG_BAD_ARGUMENT, "null system");
    if (n_basis) *n_basis = s->d.n_basis;
    if (n_occupied) *n_occupied = s->d.n_occ;
    if (n_pairs) *n_pairs = s->d.n_pairs;
    return PDG_OK;
}

static FramePlan plan_for(const pdg_system *s, int history) { return make_plan(s->d, history < 1 ? 1 : history); }

extern "C" size_t pdg_workspace_bytes(const pdg_system *s, int n_frames)
{
    if (!s || n_frames <= 0) return 0;
    return sizeof(double) * plan_for(s, PDG_MAX_HISTORY).stride * (size_t)n_frames;
}

static int check_workspace(const pdg_system *s, int n_frames, void *ws, size_t bytes)
{
    if (!s) return fail(PDG_BAD_ARGUMENT, "null system");
    if (s->d.n_electrons % 2) return fail(PDG_BAD_ARGUMENT, "closed-shell RHF needs an even electron count (odd counts: pdg_energy_gradients_uhf)");
    if (n_frames <= 0) return fail(PDG_BAD_ARGUMENT, "n_frames must be positive");
    if (!ws || bytes < pdg_workspace_bytes(s, n_frames)) return fail(PDG_BAD_ARGUMENT, "workspace missing or too small");
    return PDG_OK;
}

static int integrals(const DeviceSystem &d, const FramePlan &p, int n_frames, const double *xyz, double *ws, cudaStream_t st)
{
    launch_pair_integrals(d, p, n_frames, xyz, ws, st);
    launch_assemble_h(d, p, n_frames, ws, st);
    return cuda_check(cudaGetLastError(), "integral kernels");
}

// The system as the mixed method's kernels see it: with the tabulated overlap sums attached.
static DeviceSystem mixed_view(const pdg_system *s, bool mixed)
{
    DeviceSystem d = s->d;
    if (mixed) d.ovl_tab = s->d_ovl_tab;
    return d;
}

extern "C" int pdg_energy_gradients(pdg_system *s, int n_frames, const double *d_xyz, const double *d_phi,
                                    const pdg_scf_options *o, double *d_density, int use_density,
                                    double *d_energies, double *d_gradients, double *d_charges, int *d_status,
                                    int *d_ncycles, void *ws, size_t bytes, void *stream)
{
    int rc = check_workspace(s, n_frames, ws, bytes);
    if (rc) return rc;
    if (!o || !d_xyz || !d_density || !d_energies || !d_status) return fail(PDG_BAD_ARGUMENT, "null argument");
    if (o->history < 1 || o->history > PDG_MAX_HISTORY) return fail(PDG_BAD_ARGUMENT, "history must be 1..16");
    if (o->maximum_scf_cycles < 0) return fail(PDG_BAD_ARGUMENT, "maximum_scf_cycles must be >= 0");
    if (o->density_step != 0 && o->density_step != 3 && o->density_step != 6) return fail(PDG_BAD_ARGUMENT, "density_step must be 0, 3 or 6");
    if (use_density < 0 || use_density > 2) return fail(PDG_BAD_ARGUMENT, "use_density must be 0, 1 or 2");
    cudaStream_t st = (cudaStream_t)stream;
    FramePlan p = plan_for(s, PDG_MAX_HISTORY);
    double *w = (double *)ws;
    auto mark = [&](int k) { if (s->ev_on) cudaEventRecord(s->ev[k], st); };
    s->ev_recorded = 0;
    mark(0);
    // with a side stream: what it holds so far (the QC/MM potentials) runs beside the integrals, the SCF waits for
    // it, and what the caller queues on it next (the QC/MM gradients) waits for the SCF
    if (s->side && (rc = cuda_check(cudaEventRecord(s->side_in, s->side), "side stream event"))) return rc;
    if ((rc = integrals(mixed_view(s, o->density_step != 0), p, n_frames, d_xyz, w, st))) return rc;
    mark(1);
    if (s->side && (rc = cuda_check(cudaStreamWaitEvent(st, s->side_in, 0), "side stream wait"))) return rc;
    launch_scf(s->d, p, n_frames, d_phi, *o, d_density, use_density, d_energies, d_charges, d_status, d_ncycles, w, 0, nullptr, st,
               o->density_step != 0 ? s->shared_base : nullptr);
    if ((rc = cuda_check(cudaGetLastError(), "scf kernel"))) return rc;
    if (s->side) {
        if ((rc = cuda_check(cudaEventRecord(s->scf_out, st), "side stream event"))) return rc;
        if ((rc = cuda_check(cudaStreamWaitEvent(s->side, s->scf_out, 0), "side stream wait"))) return rc;
    }
    mark(2);
    if (d_gradients) {
        // the mixed method takes the sp-sp pair gradient terms in FP32 (assembled and summed in FP64)
        launch_pair_gradients(mixed_view(s, o->density_step != 0), p, n_frames, d_xyz, d_density, w, st, o->density_step != 0);
        launch_reduce_gradients(s->d, p, n_frames, w, d_gradients, st);
        if ((rc = cuda_check(cudaGetLastError(), "gradient kernels"))) return rc;
    }
    mark(3);
    s->ev_recorded = s->ev_on;
    return PDG_OK;
}

extern "C" int pdg_phase_events(pdg_system *s, int enable)
{
    if (!s) return fail(PDG_BAD_ARGUMENT, "null system");
    if (enable && !s->ev[0])
        for (cudaEvent_t &e : s->ev)
            if ((e = nullptr, cudaEventCreate(&e)) != cudaSuccess) return cuda_check(cudaGetLastError(), "phase events");
    s->ev_on = enable ? 1 : 0;
    s->ev_recorded = 0;
    return PDG_OK;
}

extern "C" int pdg_phase_times(const pdg_system *s, float *h_ms)
{
    if (!s || !h_ms) return fail(PDG_BAD_ARGUMENT, "null argument");
    if (!s->ev_recorded) return fail(PDG_BAD_ARGUMENT, "pdg_phase_times: no pdg_energy_gradients call recorded phase events");
    int rc = cuda_check(cudaEventSynchronize(s->ev[3]), "phase events");
    for (int k = 0; k < 3 && !rc; k++) rc = cuda_check(cudaEventElapsedTime(h_ms + k, s->ev[k], s->ev[k + 1]), "phase events");
    return rc;
}

extern "C" int pdg_wide_create(pdg_system *s, pdg_wide **out)
{
    if (s && s->d.n_electrons % 2) return fail(PDG_BAD_ARGUMENT, "closed-shell RHF needs an even electron count");
    if (!s || !out) return fail(PDG_BAD_ARGUMENT, "null argument");
    if (s->d.n_basis < 3) return fail(PDG_BAD_ARGUMENT, "pdg_wide_create: the wide engine needs at least 3 basis functions");
    int rc = wide_create(s->d, out);
    if (rc) return fail(rc, "pdg_wide_create: cuBLAS handle");
    return PDG_OK;
}

extern "C" int pdg_wide_destroy(pdg_wide *w)
{
    wide_destroy(w);
    return PDG_OK;
}

extern "C" int pdg_wide_phase_events(pdg_wide *w, int enable)
{
    if (!w) return fail(PDG_BAD_ARGUMENT, "null argument");
    return wide_timing(w, enable) ? fail(PDG_CUDA_ERROR, "pdg_wide_phase_events: event creation failed") : PDG_OK;
}

extern "C" int pdg_wide_phase_times(pdg_wide *w, float *h_ms)
{
    if (!w || !h_ms) return fail(PDG_BAD_ARGUMENT, "null argument");
    return wide_phase_times(w, h_ms);
}

extern "C" size_t pdg_wide_workspace_bytes(const pdg_system *s)
{
    return s ? wide_workspace_bytes(s->d) : 0;
}

extern "C" int pdg_wide_energy_gradients(pdg_wide *w, const double *d_xyz, const double *d_phi, const pdg_scf_options *o,
                                         double *d_density, int use_density, double *d_energies, double *d_gradients, double *d_charges,
                                         int *d_status, int *d_ncycles, void *ws, size_t bytes, void *stream)
{
    if (!w || !o || !d_xyz || !d_density || !d_energies || !d_status) return fail(PDG_BAD_ARGUMENT, "null argument");
    if (o->history < 1 || o->history > PDG_MAX_HISTORY) return fail(PDG_BAD_ARGUMENT, "history must be 1..16");
    if (o->maximum_scf_cycles < 0) return fail(PDG_BAD_ARGUMENT, "maximum_scf_cycles must be >= 0");
    if (!ws || (uintptr_t)ws % 256) return fail(PDG_BAD_ARGUMENT, "wide workspace missing or not 256-byte aligned");
    if (bytes < wide_workspace_size(w)) return fail(PDG_BAD_ARGUMENT, "wide workspace too small");
    const int rc = wide_energy_gradients(w, d_xyz, d_phi, *o, d_density, use_density, d_energies, d_gradients, d_charges, d_status,
                                         d_ncycles, (double *)ws, (cudaStream_t)stream);
    if (rc) return fail(rc, "pdg_wide_energy_gradients: a kernel, a cuBLAS call or a stream wait failed");
    return cuda_check(cudaGetLastError(), "wide SCF");
}

extern "C" int pdg_scf(pdg_system *s, int n_frames, const double *d_phi, const pdg_scf_options *o, double *d_density,
                       int use_density, double *d_energies, double *d_charges, int *d_status, int *d_ncycles,
                       void *ws, size_t bytes, void *stream)
{
    int rc = check_workspace(s, n_frames, ws, bytes);
    if (rc) return rc;
    if (!o || !d_density || !d_energies || !d_status) return fail(PDG_BAD_ARGUMENT, "null argument");
    if (o->history < 1 || o->history > PDG_MAX_HISTORY) return fail(PDG_BAD_ARGUMENT, "history must be 1..16");
    if (o->maximum_scf_cycles < 0) return fail(PDG_BAD_ARGUMENT, "maximum_scf_cycles must be >= 0");
    if (o->density_step != 0 && o->density_step != 3 && o->density_step != 6) return fail(PDG_BAD_ARGUMENT, "density_step must be 0, 3 or 6");
    if (use_density < 0 || use_density > 2) return fail(PDG_BAD_ARGUMENT, "use_density must be 0, 1 or 2");
    FramePlan p = plan_for(s, PDG_MAX_HISTORY);
    launch_scf(s->d, p, n_frames, d_phi, *o, d_density, use_density, d_energies, d_charges, d_status, d_ncycles, (double *)ws, 0,
               nullptr, (cudaStream_t)stream, o->density_step != 0 ? s->shared_base : nullptr);
    return cuda_check(cudaGetLastError(), "scf kernel");
}

// ---- open-shell (UHF) and fractional-occupancy energies and gradients
// The frame plan of the open-shell / fractional-occupancy SCF: room for every eigenpair of a set's matrix.
static FramePlan open_plan(const pdg_system *s)
{
    DeviceSystem d = s->d;
    d.n_vec = d.n_basis;
    return make_plan(d, PDG_MAX_HISTORY);
}

extern "C" size_t pdg_open_workspace_bytes(pdg_system *s, int n_frames)
{
    if (!s || n_frames <= 0) return 0;
    return 2 * (size_t)n_frames * open_plan(s).stride * sizeof(double);
}

extern "C" size_t pdg_uhf_workspace_bytes(pdg_system *s, int n_frames, int n_alpha, int n_beta)
{
    (void)n_alpha; (void)n_beta;
    return pdg_open_workspace_bytes(s, n_frames);
}

// One density set's occupancies by occupancy_init's rules (QCOnePDM.c:290-330, with the orbital checks of
// QCModel.CrossCheckModelAndState, pMolecule.QCModel.pyx:119-135): cardinal needs a whole number of full orbitals;
// fixed fractional spreads the charge left over by the nOcc - nHOO full orbitals evenly over nHOO + nLUO orbitals.
static bool occupancy_set(int type, double factor, double charge, int nHOO, int nLUO, int N, OpenOccupancy &oc, int q)
{
    if (!(charge >= 0.0)) return false;
    const int nocc = (int)std::lround(std::ceil(charge / factor));
    if (nocc > N) return false;
    int ncard = 0, nfrac = 0;
    double frac = 0.0;
    bool ok = true;
    if (type == PDG_OCC_CARDINAL) { ok = std::fabs(nocc * factor - charge) < 1.0e-10; ncard = nocc; }
    else if (type == PDG_OCC_FIXED_FRACTIONAL) {
        ncard = nocc - nHOO; nfrac = nHOO + nLUO;
        frac = (charge / factor - ncard) / (double)std::max(nfrac, 1);
        ok = nHOO > 0 && nLUO >= 0 && ncard >= 0 && ncard + nfrac <= N && frac >= 0.0 && frac <= 1.0;
    }
    oc.charge[q] = charge; oc.ncard[q] = ncard; oc.nfrac[q] = nfrac; oc.frac[q] = frac;
    return ok;
}

extern "C" int pdg_energy_gradients_open(pdg_system *s, int n_frames, const double *d_xyz, const double *d_phi, const pdg_scf_options *o,
                                         const pdg_occupancy *occ, double *d_density, int use_density, double *d_energies,
                                         double *d_gradients, double *d_charges, int *d_status, int *d_ncycles, double *d_total_spin,
                                         void *ws, size_t bytes, void *stream)
{
    if (!s || n_frames <= 0) return fail(PDG_BAD_ARGUMENT, "pdg_energy_gradients_open: bad argument");
    if (!o || !occ || !d_xyz || !d_density || !d_energies || !d_status)
        return fail(PDG_BAD_ARGUMENT, "pdg_energy_gradients_open: null argument");
    if (o->history < 1 || o->history > PDG_MAX_HISTORY) return fail(PDG_BAD_ARGUMENT, "history must be 1..16");
    if (o->maximum_scf_cycles < 0) return fail(PDG_BAD_ARGUMENT, "maximum_scf_cycles must be >= 0");
    if (o->density_step != 0) return fail(PDG_BAD_ARGUMENT, "pdg_energy_gradients_open: the FP64 density step only (density_step 0)");
    if (use_density < 0 || use_density > 2) return fail(PDG_BAD_ARGUMENT, "use_density must be 0, 1 or 2");
    const int N = s->d.n_basis;
    OpenOccupancy oc = {};
    oc.type = occ->occupancy_type;
    if (oc.type < PDG_OCC_CARDINAL || oc.type > PDG_OCC_VARIABLE_FRACTIONAL) return fail(PDG_BAD_ARGUMENT, "unknown occupancy type");
    const double a = occ->alpha_charge, b = occ->beta_charge;
    if (!(a >= 0.0) || !(b >= 0.0) || std::fabs(a + b - (double)s->d.n_electrons) > 1.0e-10)
        return fail(PDG_BAD_ARGUMENT, "alpha and beta charges must be >= 0 and add up to the electrons");
    if (oc.type == PDG_OCC_VARIABLE_FRACTIONAL && !(occ->fermi_broadening > 0.0))
        return fail(PDG_BAD_ARGUMENT, "the Fermi broadening must be > 0");
    oc.beta = occ->fermi_broadening;
    const int *nf = occ->n_fractional;
    bool ok;
    if (occ->spin_restricted) {
        oc.n_sets = 1; oc.factor = 2.0;
        ok = occupancy_set(oc.type, 2.0, a + b, nf[0], nf[1], N, oc, 0);
    } else {
        oc.n_sets = 2; oc.factor = 1.0;
        ok = occupancy_set(oc.type, 1.0, a, nf[2], nf[3], N, oc, 0) && occupancy_set(oc.type, 1.0, b, nf[4], nf[5], N, oc, 1);
    }
    if (!ok) return fail(PDG_BAD_ARGUMENT, "invalid occupancies (orbital counts, fractional orbital specification or charges)");
    if (d_gradients && oc.n_sets == 2 && !d_total_spin) return fail(PDG_BAD_ARGUMENT, "pdg_energy_gradients_open: null d_total_spin");
    if (!ws || bytes < pdg_open_workspace_bytes(s, n_frames)) return fail(PDG_BAD_ARGUMENT, "workspace missing or too small");
    cudaStream_t st = (cudaStream_t)stream;
    const FramePlan p = open_plan(s);
    double *w = (double *)ws;
    int rc;
    if ((rc = integrals(s->d, p, n_frames, d_xyz, w, st))) return rc;
    launch_scf_open(s->d, p, n_frames, d_phi, *o, oc, d_density, use_density, d_energies, d_charges, d_status, d_ncycles, w, st);
    if ((rc = cuda_check(cudaGetLastError(), "open-shell scf kernel"))) return rc;
    if (d_gradients) {
        if (oc.n_sets == 2) {
            launch_uhf_densities(n_frames, N, d_density, d_total_spin, st);
            DeviceSystem dg = s->d;
            dg.spin = d_total_spin + (size_t)n_frames * N * N;
            launch_pair_gradients(dg, p, n_frames, d_xyz, d_total_spin, w, st, false);
        } else {
            launch_pair_gradients(s->d, p, n_frames, d_xyz, d_density, w, st, false);
        }
        launch_reduce_gradients(s->d, p, n_frames, w, d_gradients, st);
        if ((rc = cuda_check(cudaGetLastError(), "gradient kernels"))) return rc;
    }
    return PDG_OK;
}

extern "C" int pdg_energy_gradients_uhf(pdg_system *s, int n_frames, const double *d_xyz, const double *d_phi, const pdg_scf_options *o,
                                        int n_alpha, int n_beta, double *d_density, int use_density, double *d_energies,
                                        double *d_gradients, double *d_charges, int *d_status, int *d_ncycles, double *d_total_spin,
                                        void *ws, size_t bytes, void *stream)
{
    if (!s) return fail(PDG_BAD_ARGUMENT, "pdg_energy_gradients_uhf: bad argument");
    if (n_alpha < n_beta || n_beta < 0 || n_alpha > s->d.n_basis || n_alpha + n_beta != s->d.n_electrons)
        return fail(PDG_BAD_ARGUMENT, "pdg_energy_gradients_uhf: n_alpha >= n_beta >= 0, n_alpha <= N and n_alpha + n_beta = the electrons");
    pdg_occupancy occ = {};
    occ.spin_restricted = 0; occ.occupancy_type = PDG_OCC_CARDINAL;
    occ.alpha_charge = n_alpha; occ.beta_charge = n_beta;
    return pdg_energy_gradients_open(s, n_frames, d_xyz, d_phi, o, &occ, d_density, use_density, d_energies, d_gradients, d_charges,
                                     d_status, d_ncycles, d_total_spin, ws, bytes, stream);
}

// ---- shared base of the mixed method's perturbative density steps
extern "C" size_t pdg_base_bytes(pdg_system *s)
{
    if (!s) return 0;
    const FramePlan p = plan_for(s, PDG_MAX_HISTORY);
    return (p.stride - p.BF) * sizeof(double);
}

extern "C" int pdg_base_capture(pdg_system *s, int n_frames, int frame, const void *ws, size_t bytes, void *d_base, void *stream)
{
    int rc = check_workspace(s, n_frames, const_cast<void *>(ws), bytes);
    if (rc) return rc;
    if (frame < 0 || frame >= n_frames || !d_base) return fail(PDG_BAD_ARGUMENT, "pdg_base_capture: bad argument");
    if ((uintptr_t)d_base % 16) return fail(PDG_BAD_ARGUMENT, "pdg_base_capture: base not 16-byte aligned");
    const FramePlan p = plan_for(s, PDG_MAX_HISTORY);
    const double *src = (const double *)ws + (size_t)frame * p.stride + p.BF;
    return cuda_check(cudaMemcpyAsync(d_base, src, (p.stride - p.BF) * sizeof(double), cudaMemcpyDeviceToDevice, (cudaStream_t)stream),
                      "pdg_base_capture copy");
}

extern "C" int pdg_set_side_stream(pdg_system *s, void *side_stream)
{
    if (!s) return fail(PDG_BAD_ARGUMENT, "null system");
    if (side_stream && !s->side_in) {
        if (cudaEventCreateWithFlags(&s->side_in, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&s->scf_out, cudaEventDisableTiming) != cudaSuccess)
            return cuda_check(cudaGetLastError(), "side stream events");
    }
    s->side = (cudaStream_t)side_stream;
    return PDG_OK;
}

extern "C" int pdg_set_shared_base(pdg_system *s, const void *d_base)
{
    if (!s) return fail(PDG_BAD_ARGUMENT, "null system");
    if ((uintptr_t)d_base % 16) return fail(PDG_BAD_ARGUMENT, "pdg_set_shared_base: base not 16-byte aligned");
    s->shared_base = (const double *)d_base;
    return PDG_OK;
}

extern "C" int pdg_one_electron(pdg_system *s, int n_frames, const double *d_xyz, double *d_h, void *ws, size_t bytes, void *stream)
{
    int rc = check_workspace(s, n_frames, ws, bytes);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    FramePlan p = plan_for(s, PDG_MAX_HISTORY);
    double *w = (double *)ws;
    if ((rc = integrals(s->d, p, n_frames, d_xyz, w, st))) return rc;
    size_t NN = (size_t)s->d.n_basis * s->d.n_basis;
    for (int f = 0; f < n_frames; f++)
        if ((rc = cuda_check(cudaMemcpyAsync(d_h + f * NN, w + f * p.stride + p.H, sizeof(double) * NN, cudaMemcpyDeviceToDevice, st), "copy H"))) return rc;
    return PDG_OK;
}

extern "C" int pdg_fock(pdg_system *s, int n_frames, const double *d_xyz, const double *d_phi, const double *d_density,
                        double *d_fock, double *d_energies, void *ws, size_t bytes, void *stream)
{
    int rc = check_workspace(s, n_frames, ws, bytes);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    FramePlan p = plan_for(s, PDG_MAX_HISTORY);
    double *w = (double *)ws;
    if ((rc = integrals(s->d, p, n_frames, d_xyz, w, st))) return rc;
    pdg_scf_options o = { 1e-8, 2e-4, 0.2, 0, 10, 1, 0, 1e-4 };
    launch_scf(s->d, p, n_frames, d_phi, o, const_cast<double *>(d_density), 1, d_energies, nullptr, nullptr, nullptr, w, 1, d_fock, st);
    return cuda_check(cudaGetLastError(), "fock kernel");
}

extern "C" int pdg_gradients(pdg_system *s, int n_frames, const double *d_xyz, const double *d_density,
                             double *d_gradients, void *ws, size_t bytes, void *stream)
{
    int rc = check_workspace(s, n_frames, ws, bytes);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    FramePlan p = plan_for(s, PDG_MAX_HISTORY);
    double *w = (double *)ws;
    launch_pair_gradients(s->d, p, n_frames, d_xyz, d_density, w, st);
    launch_reduce_gradients(s->d, p, n_frames, w, d_gradients, st);
    return cuda_check(cudaGetLastError(), "gradient kernels");
}

extern "C" int pdg_scf_timings(const pdg_system *s, int n_frames, const void *ws, size_t bytes, double *d_out, void *stream)
{
    int rc = check_workspace(s, n_frames, const_cast<void *>(ws), bytes);
    if (rc) return rc;
    if (!d_out) return fail(PDG_BAD_ARGUMENT, "null output");
    FramePlan p = plan_for(s, PDG_MAX_HISTORY);
    const double *w = (const double *)ws;
    cudaStream_t st = (cudaStream_t)stream;
    for (int f = 0; f < n_frames; f++)
        if ((rc = cuda_check(cudaMemcpyAsync(d_out + (size_t)f * PDG_NTIMERS, w + f * p.stride + p.misc + PDG_MAX_HISTORY * PDG_MAX_HISTORY,
                                             sizeof(double) * PDG_NTIMERS, cudaMemcpyDeviceToDevice, st), "copy timings"))) return rc;
    return PDG_OK;
}

extern "C" size_t pdg_qcmm_workspace_bytes(int n_frames, int n_mm)
{
    if (n_frames <= 0 || n_mm < 0) return 0;
    return qcmm_workspace_bytes(n_frames, n_mm);
}

static int check_qcmm_workspace(int n_frames, int n_mm, void *ws, size_t bytes)
{
    if (!ws || bytes < qcmm_workspace_bytes(n_frames, n_mm)) return fail(PDG_BAD_ARGUMENT, "QC/MM workspace missing or too small");
    if ((uintptr_t)ws % 256) return fail(PDG_BAD_ARGUMENT, "QC/MM workspace must be 256-byte aligned");
    return PDG_OK;
}

extern "C" int pdg_qcmm_potentials(int model, int n_frames, int n_qc, int n_mm, const double *qc, const double *mm,
                                   const double *q, int n_knots, const double *knots, double cutoff, double *phi,
                                   void *ws, size_t bytes, void *stream)
{
    if (model != 0 && model != 1) return fail(PDG_BAD_ARGUMENT, "model must be 0 (full) or 1 (ABFS)");
    if (n_frames <= 0 || n_qc <= 0 || n_mm < 0 || !qc || !phi || (n_mm > 0 && (!mm || !q))) return fail(PDG_BAD_ARGUMENT, "bad sizes or null pointers");
    if (n_qc > PDG_MAX_ATOMS) return fail(PDG_TOO_LARGE, "more QC atoms than PDG_MAX_ATOMS");
    if (model == 1 && (n_knots < 2 || !knots || cutoff <= 0.0)) return fail(PDG_BAD_ARGUMENT, "ABFS needs spline knots and a cutoff");
    int rc = check_qcmm_workspace(n_frames, n_mm, ws, bytes);
    if (rc) return rc;
    launch_qcmm_potentials(model, n_frames, n_qc, n_mm, qc, mm, q, n_knots, knots, cutoff, phi, ws, (cudaStream_t)stream);
    return cuda_check(cudaGetLastError(), "qcmm potentials");
}

extern "C" int pdg_qcmm_gradients(int model, int n_frames, int n_qc, int n_mm, const double *qc, const double *mm,
                                  const double *q, const double *qcq, int n_knots, const double *knots, double cutoff,
                                  double *gqc, double *gmm, void *ws, size_t bytes, void *stream)
{
    const int base_model = model & ~PDG_QCMM_FP32_PAIRS;
    if ((base_model != 0 && base_model != 1) || (model & ~(PDG_QCMM_FP32_PAIRS | 1))) return fail(PDG_BAD_ARGUMENT, "model must be 0 (full) or 1 (ABFS), optionally | PDG_QCMM_FP32_PAIRS");
    if (model & PDG_QCMM_FP32_PAIRS && base_model == 1 && n_knots > 1024) return fail(PDG_TOO_LARGE, "FP32 pair terms take at most 1024 spline knots");
    if (n_frames <= 0 || n_qc <= 0 || n_mm < 0 || !qc || !qcq || !gqc || (n_mm > 0 && (!mm || !q))) return fail(PDG_BAD_ARGUMENT, "bad sizes or null pointers");
    if (n_qc > PDG_MAX_ATOMS) return fail(PDG_TOO_LARGE, "more QC atoms than PDG_MAX_ATOMS");
    if (base_model == 1 && (n_knots < 2 || !knots || cutoff <= 0.0)) return fail(PDG_BAD_ARGUMENT, "ABFS needs spline knots and a cutoff");
    int rc = check_qcmm_workspace(n_frames, n_mm, ws, bytes);
    if (rc) return rc;
    launch_qcmm_gradients(model, n_frames, n_qc, n_mm, qc, mm, q, qcq, n_knots, knots, cutoff, gqc, gmm, ws, (cudaStream_t)stream);
    return cuda_check(cudaGetLastError(), "qcmm gradients");
}

// ---------------------------------------------------------------------------------------------------
// Gradients with library-owned scratch: pdg_gradients without a caller workspace and without any device
// allocation at call time, for callers that may not allocate (declared in include/pdg.h).  The scratch
// is a file-scope device array; every device has its own instance, whose address is looked up once per
// device and cached.  It holds the per-pair gradient terms, n_frames * n_pairs * 3 doubles; each element
// the reduction reads is written earlier in the same call, so nothing needs to start at zero.
#define PDG_STATIC_SCRATCH_DOUBLES (512 * 1024)
#define PDG_STATIC_MAX_DEVICES 64
static __device__ __align__(256) double g_static_scratch[PDG_STATIC_SCRATCH_DOUBLES];
static std::mutex g_static_mutex;
static double *g_static_ptr[PDG_STATIC_MAX_DEVICES] = {};

extern "C" int pdg_gradients_static_scratch(pdg_system *s, int n_frames, const double *d_xyz, const double *d_density,
                                            double *d_gradients, void *stream)
{
    if (!s) return fail(PDG_BAD_ARGUMENT, "null system");
    if (n_frames <= 0) return fail(PDG_BAD_ARGUMENT, "n_frames must be positive");
    if (!d_xyz || !d_density || !d_gradients) return fail(PDG_BAD_ARGUMENT, "null argument");
    FramePlan p = {};
    p.pair_g = 0;
    p.stride = align32((size_t)s->d.n_pairs * 3);
    const size_t need = p.stride * (size_t)n_frames;
    if (need > PDG_STATIC_SCRATCH_DOUBLES)
        return fail(PDG_TOO_LARGE, "pdg_gradients_static_scratch: " + std::to_string(n_frames) + " frames of " +
                                       std::to_string(s->d.n_pairs) + " atom pairs need " + std::to_string(need) +
                                       " doubles of scratch, more than the " + std::to_string(PDG_STATIC_SCRATCH_DOUBLES) +
                                       " compiled in; use pdg_gradients with a workspace");
    int dev = 0, rc;
    if ((rc = cuda_check(cudaGetDevice(&dev), "cudaGetDevice"))) return rc;
    if (dev < 0 || dev >= PDG_STATIC_MAX_DEVICES) return fail(PDG_TOO_LARGE, "device ordinal beyond 63");
    double *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_static_mutex);
        if (!g_static_ptr[dev]) {
            void *ptr = nullptr;
            if ((rc = cuda_check(cudaGetSymbolAddress(&ptr, g_static_scratch), "cudaGetSymbolAddress (static scratch)"))) return rc;
            g_static_ptr[dev] = (double *)ptr;
        }
        scratch = g_static_ptr[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    launch_pair_gradients(s->d, p, n_frames, d_xyz, d_density, scratch, st);
    launch_reduce_gradients(s->d, p, n_frames, scratch, d_gradients, st);
    return cuda_check(cudaGetLastError(), "gradient kernels (static scratch)");
}

extern "C" int pdg_tc_selftest(int n, int kprod, int wait_limit, const float *d_x, float *d_c, int *d_status, void *stream)
{
    if (kprod != 0 && kprod != 1 && kprod != 3 && kprod != 6) return fail(PDG_BAD_ARGUMENT, "pdg_tc_selftest: kprod must be 0, 1, 3 or 6");
    if (!d_status) return fail(PDG_BAD_ARGUMENT, "null argument");
    if (kprod != 0) {
        if (n < 1 || n > 144) return fail(PDG_TOO_LARGE, "pdg_tc_selftest: n must be 1..144");
        if (!d_x || !d_c) return fail(PDG_BAD_ARGUMENT, "null argument");
    }
    launch_tc_selftest(n, kprod, wait_limit, d_x, d_c, d_status, (cudaStream_t)stream);
    return cuda_check(cudaGetLastError(), "tensor-core self-test kernel");
}

extern "C" int pdg_density(pdg_system *s, int n_frames, const double *d_fock, int density_step, double *d_density,
                           double *d_energies, int *d_status, void *ws, size_t bytes, void *stream)
{
    int rc = check_workspace(s, n_frames, ws, bytes);
    if (rc) return rc;
    if (!d_fock || !d_density || !d_energies || !d_status) return fail(PDG_BAD_ARGUMENT, "null argument");
    if (density_step != 0 && density_step != 3 && density_step != 6) return fail(PDG_BAD_ARGUMENT, "density_step must be 0, 3 or 6");
    FramePlan p = plan_for(s, PDG_MAX_HISTORY);
    pdg_scf_options o = { 1e-8, 2e-4, 0.2, 0, 10, 1, density_step, 1e-4 };
    launch_scf(s->d, p, n_frames, nullptr, o, d_density, 1, d_energies, nullptr, d_status, nullptr, (double *)ws, 2,
               const_cast<double *>(d_fock), (cudaStream_t)stream);
    return cuda_check(cudaGetLastError(), "density step kernel");
}

extern "C" int pdg_scf_occupancy(const pdg_system *s, int *threads, int *smem_bytes, int *ctas_per_sm)
{
    if (!s || !threads || !smem_bytes || !ctas_per_sm) return fail(PDG_BAD_ARGUMENT, "null argument");
    if (scf_occupancy(s->d, threads, smem_bytes, ctas_per_sm)) return cuda_check(cudaGetLastError(), "occupancy query");
    return PDG_OK;
}

// ---------------------------------------------------------------------------------------------------
// Heterogeneous batches: independent molecules of different sizes in one launch per kernel.
struct pdg_batch {
    std::vector<BatchItem> items;   // host copy of the device table
    BatchItem *d_items = nullptr;
    int *d_order = nullptr, *d_queue = nullptr;
    Batch b = {};
    size_t ws_doubles = 0, dens_doubles = 0;
    int n_atoms = 0, sms = 0;
    // schedule (pdg_batch_schedule): SCF variant (256 or 512 threads per CTA), CTAs per SM, queue order
    int threads = 256, ctas_per_sm = 2, order_mode = 0, grid = 0, smem_limit = 0, tensor_items = 0;
    size_t smem_bytes = 0;
};

static int batch_schedule(pdg_batch *bt, int threads, int ctas_per_sm, int order_mode)
{
    const int n = bt->b.n;
    const bool wide = threads == 512;
    bt->threads = threads;
    bt->ctas_per_sm = ctas_per_sm;
    bt->order_mode = order_mode;
    bt->smem_limit = ctas_per_sm == 1 ? PDG_SMEM_LIMIT_1 : PDG_SMEM_LIMIT_2;
    bt->grid = std::max(1, std::min(n, bt->sms * ctas_per_sm));
    bt->smem_bytes = 0;
    bt->tensor_items = 0;
    for (const BatchItem &it : bt->items) {
        const size_t by = wide ? scf_w::scf_smem_bytes_limit(it.s.n_basis, it.s.n_vec, bt->smem_limit)
                               : scf_n::scf_smem_bytes_limit(it.s.n_basis, it.s.n_vec, bt->smem_limit);
        bt->smem_bytes = std::max(bt->smem_bytes, by);
        // the purification step (256-thread variant only) needs N <= 144 and the packed matrix in shared
        // memory (the plan's amat)
        const size_t small = scf_n::scf_smem_bytes_limit(it.s.n_basis, it.s.n_vec, 0);
        if (!wide && it.s.n_basis <= 144 && by > small) bt->tensor_items++;
    }
    std::vector<int> order(n);
    for (int k = 0; k < n; k++) order[k] = k;
    if (order_mode == 0)   // largest first (N^3 work), so that the last CTAs to finish hold the smallest items
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return bt->items[x].s.n_basis > bt->items[y].s.n_basis; });
    int rc;
    if ((rc = cuda_check(cudaMemcpy(bt->d_order, order.data(), sizeof(int) * n, cudaMemcpyHostToDevice), "copy batch order"))) return rc;
    if (wide ? scf_w::configure_batch_scf(bt->smem_bytes) : scf_n::configure_batch_scf(bt->smem_bytes))
        return cuda_check(cudaGetLastError(), "batch SCF launch attributes");
    return PDG_OK;
}

extern "C" int pdg_batch_create(pdg_system *const *systems, int n_items, pdg_batch **out)
{
    if (!out || !systems) return fail(PDG_BAD_ARGUMENT, "null argument");
    *out = nullptr;
    if (n_items <= 0) return fail(PDG_BAD_ARGUMENT, "n_items must be positive");
    pdg_batch *bt = new pdg_batch();
    long long ws = 0, dens = 0, atom = 0, work[PDG_WORK_KINDS] = {};
    for (int k = 0; k < n_items; k++) {
        if (!systems[k]) { delete bt; return fail(PDG_BAD_ARGUMENT, "null system in batch"); }
        if (systems[k]->d.n_electrons % 2) { delete bt; return fail(PDG_BAD_ARGUMENT, "closed-shell RHF needs an even electron count"); }
        BatchItem it = {};
        it.s = systems[k]->d;
        it.plan = plan_for(systems[k], PDG_MAX_HISTORY);
        it.ws = ws; it.dens = dens; it.atom = (int)atom;
        for (int c = 0; c < PDG_WORK_KINDS; c++) it.work[c] = (int)work[c];
        ws += (long long)it.plan.stride;
        dens += (long long)it.s.n_basis * it.s.n_basis;
        atom += it.s.n_atoms;
        for (int c = 0; c < PDG_WORK_KINDS; c++) work[c] += work_units(it.s, c);
        bt->items.push_back(it);
    }
    if (work[0] > INT32_MAX || work[1] > INT32_MAX || work[2] > INT32_MAX || work[3] > INT32_MAX || atom > INT32_MAX) {
        delete bt;
        return fail(PDG_TOO_LARGE, "batch work exceeds 2^31 units");
    }
    bt->b.n = n_items;
    for (int c = 0; c < PDG_WORK_KINDS; c++) bt->b.total[c] = (int)work[c];
    bt->ws_doubles = (size_t)ws; bt->dens_doubles = (size_t)dens; bt->n_atoms = (int)atom;
    int dev = 0, rc;
    if ((rc = cuda_check(cudaGetDevice(&dev), "cudaGetDevice")) ||
        (rc = cuda_check(cudaDeviceGetAttribute(&bt->sms, cudaDevAttrMultiProcessorCount, dev), "SM count")) ||
        (rc = cuda_check(cudaMalloc(&bt->d_items, sizeof(BatchItem) * n_items), "cudaMalloc batch table")) ||
        (rc = cuda_check(cudaMalloc(&bt->d_order, sizeof(int) * n_items), "cudaMalloc batch order")) ||
        (rc = cuda_check(cudaMalloc(&bt->d_queue, sizeof(int)), "cudaMalloc batch queue")) ||
        (rc = cuda_check(cudaMemcpy(bt->d_items, bt->items.data(), sizeof(BatchItem) * n_items, cudaMemcpyHostToDevice), "copy batch table"))) {
        pdg_batch_destroy(bt);
        return rc;
    }
    bt->b.items = bt->d_items;
    if ((rc = batch_schedule(bt, 256, 2, 0))) { pdg_batch_destroy(bt); return rc; }
    *out = bt;
    return PDG_OK;
}

extern "C" int pdg_batch_destroy(pdg_batch *bt)
{
    if (!bt) return PDG_OK;
    cudaFree(bt->d_items); cudaFree(bt->d_order); cudaFree(bt->d_queue);
    delete bt;
    return PDG_OK;
}

extern "C" int pdg_batch_info(const pdg_batch *bt, int *n_items, int *n_atoms, long long *density_doubles, int *grid, int *threads,
                              int *smem_bytes, int *tensor_items)
{
    if (!bt) return fail(PDG_BAD_ARGUMENT, "null batch");
    if (threads) *threads = bt->threads;
    if (n_items) *n_items = bt->b.n;
    if (n_atoms) *n_atoms = bt->n_atoms;
    if (density_doubles) *density_doubles = (long long)bt->dens_doubles;
    if (grid) *grid = bt->grid;
    if (smem_bytes) *smem_bytes = (int)bt->smem_bytes;
    if (tensor_items) *tensor_items = bt->tensor_items;
    return PDG_OK;
}

extern "C" size_t pdg_batch_workspace_bytes(const pdg_batch *bt) { return bt ? sizeof(double) * bt->ws_doubles : 0; }

extern "C" int pdg_batch_schedule(pdg_batch *bt, int threads, int ctas_per_sm, int order)
{
    if (!bt) return fail(PDG_BAD_ARGUMENT, "null batch");
    if (!((threads == 256 && (ctas_per_sm == 1 || ctas_per_sm == 2)) || (threads == 512 && ctas_per_sm == 1)))
        return fail(PDG_BAD_ARGUMENT, "schedule must be 256 threads with 1 or 2 CTAs per SM, or 512 threads with 1");
    if (order != 0 && order != 1) return fail(PDG_BAD_ARGUMENT, "order must be 0 (largest first) or 1 (item order)");
    return batch_schedule(bt, threads, ctas_per_sm, order);
}

static int batch_queue(pdg_batch *bt, const double *d_xyz, const double *d_phi, const pdg_scf_options *o, double *d_density,
                       int use_density, double *d_energies, double *d_gradients, double *d_charges, int *d_status, int *d_ncycles,
                       void *ws, cudaStream_t st)
{
    double *w = (double *)ws;
    int rc;
    launch_batch_integrals(bt->b, d_xyz, w, st);
    if ((rc = cuda_check(cudaGetLastError(), "batch integral kernels"))) return rc;
    if ((rc = cuda_check(cudaMemsetAsync(bt->d_queue, 0, sizeof(int), st), "reset batch queue"))) return rc;
    if (bt->threads == 512)
        scf_w::launch_batch_scf(bt->b, bt->d_order, bt->d_queue, bt->grid, bt->smem_limit, bt->smem_bytes, 0, d_phi, *o, d_density,
                                use_density, d_energies, d_charges, d_status, d_ncycles, w, st);
    else
        scf_n::launch_batch_scf(bt->b, bt->d_order, bt->d_queue, bt->grid, bt->smem_limit, bt->smem_bytes, bt->tensor_items, d_phi, *o,
                                d_density, use_density, d_energies, d_charges, d_status, d_ncycles, w, st);
    if ((rc = cuda_check(cudaGetLastError(), "batch scf kernel"))) return rc;
    if (d_gradients) {
        launch_batch_gradients(bt->b, d_xyz, d_density, w, d_gradients, st, o->density_step != 0);
        if ((rc = cuda_check(cudaGetLastError(), "batch gradient kernels"))) return rc;
    }
    return PDG_OK;
}

static int batch_check(const pdg_batch *bt, const double *d_xyz, const pdg_scf_options *o, const double *d_density,
                       const double *d_energies, const int *d_status, const void *ws, size_t bytes)
{
    if (!bt) return fail(PDG_BAD_ARGUMENT, "null batch");
    if (!o || !d_xyz || !d_density || !d_energies || !d_status) return fail(PDG_BAD_ARGUMENT, "null argument");
    if (!ws || bytes < pdg_batch_workspace_bytes(bt)) return fail(PDG_BAD_ARGUMENT, "workspace missing or too small");
    if (o->history < 1 || o->history > PDG_MAX_HISTORY) return fail(PDG_BAD_ARGUMENT, "history must be 1..16");
    if (o->maximum_scf_cycles < 0) return fail(PDG_BAD_ARGUMENT, "maximum_scf_cycles must be >= 0");
    if (o->density_step != 0 && o->density_step != 3 && o->density_step != 6) return fail(PDG_BAD_ARGUMENT, "density_step must be 0, 3 or 6");
    return PDG_OK;
}

extern "C" int pdg_batch_energy_gradients(pdg_batch *bt, const double *d_xyz, const double *d_phi, const pdg_scf_options *o,
                                          double *d_density, int use_density, double *d_energies, double *d_gradients,
                                          double *d_charges, int *d_status, int *d_ncycles, void *ws, size_t bytes, void *stream)
{
    int rc = batch_check(bt, d_xyz, o, d_density, d_energies, d_status, ws, bytes);
    if (rc) return rc;
    return batch_queue(bt, d_xyz, d_phi, o, d_density, use_density, d_energies, d_gradients, d_charges, d_status, d_ncycles, ws,
                       (cudaStream_t)stream);
}

extern "C" int pdg_batch_timings(const pdg_batch *bt, const void *ws, size_t bytes, double *d_out, void *stream)
{
    if (!bt || !d_out) return fail(PDG_BAD_ARGUMENT, "null argument");
    if (!ws || bytes < pdg_batch_workspace_bytes(bt)) return fail(PDG_BAD_ARGUMENT, "workspace missing or too small");
    const double *w = (const double *)ws;
    int rc;
    for (int k = 0; k < bt->b.n; k++) {
        const BatchItem &it = bt->items[k];
        if ((rc = cuda_check(cudaMemcpyAsync(d_out + (size_t)k * PDG_NTIMERS, w + it.ws + it.plan.misc + PDG_MAX_HISTORY * PDG_MAX_HISTORY,
                                             sizeof(double) * PDG_NTIMERS, cudaMemcpyDeviceToDevice, (cudaStream_t)stream), "copy timings")))
            return rc;
    }
    return PDG_OK;
}

struct pdg_graph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

extern "C" int pdg_batch_graph_create(pdg_batch *bt, const double *d_xyz, const double *d_phi, const pdg_scf_options *o,
                                      double *d_density, int use_density, double *d_energies, double *d_gradients,
                                      double *d_charges, int *d_status, int *d_ncycles, void *ws, size_t bytes, pdg_graph **out)
{
    if (!out) return fail(PDG_BAD_ARGUMENT, "null argument");
    *out = nullptr;
    int rc = batch_check(bt, d_xyz, o, d_density, d_energies, d_status, ws, bytes);
    if (rc) return rc;
    cudaStream_t st = nullptr;
    if ((rc = cuda_check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "capture stream"))) return rc;
    pdg_graph *g = new pdg_graph();
    rc = cuda_check(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
    if (!rc) {
        const int qr = batch_queue(bt, d_xyz, d_phi, o, d_density, use_density, d_energies, d_gradients, d_charges, d_status, d_ncycles,
                                   ws, st);
        const int er = cuda_check(cudaStreamEndCapture(st, &g->graph), "end capture");
        rc = qr ? qr : er;
    }
    if (!rc) rc = cuda_check(cudaGraphInstantiate(&g->exec, g->graph, 0), "instantiate graph");
    cudaStreamDestroy(st);
    if (rc) { pdg_graph_destroy(g); return rc; }
    *out = g;
    return PDG_OK;
}

extern "C" int pdg_graph_launch(pdg_graph *g, void *stream)
{
    if (!g || !g->exec) return fail(PDG_BAD_ARGUMENT, "null graph");
    return cuda_check(cudaGraphLaunch(g->exec, (cudaStream_t)stream), "graph launch");
}

extern "C" int pdg_graph_destroy(pdg_graph *g)
{
    if (!g) return PDG_OK;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    return PDG_OK;
}

// ---------------------------------------------------------------------------------------------------
// Learned start density (guess.cu)
extern "C" int pdg_guess_features(pdg_system *s, int n_frames, const double *d_xyz, const double *d_phi, float *d_env, int *d_count,
                                  int *d_offsets, float *d_x, int *d_row_frame, int *d_row_pair, void *stream)
{
    if (!s || n_frames <= 0 || !d_xyz || !d_env || !d_count || !d_offsets || !d_x || !d_row_frame || !d_row_pair)
        return fail(PDG_BAD_ARGUMENT, "pdg_guess_features: bad argument");
    launch_guess_features(s->d, n_frames, d_xyz, d_phi, d_env, d_count, d_offsets, d_x, d_row_frame, d_row_pair, (cudaStream_t)stream);
    return cuda_check(cudaGetLastError(), "guess feature kernels");
}

extern "C" int pdg_mlp_forward(int max_rows, const int *d_rows, int k, int n, const float *d_x, const void *d_w, const float *d_b,
                               float *d_z, float *d_h, int act, void *stream)
{
    if (max_rows <= 0 || !d_rows || k <= 0 || n <= 0 || !d_x || !d_w || !d_b || !d_h) return fail(PDG_BAD_ARGUMENT, "pdg_mlp_forward: bad argument");
    launch_mlp_forward(max_rows, d_rows, k, n, d_x, d_w, d_b, d_z, d_h, act, (cudaStream_t)stream);
    return cuda_check(cudaGetLastError(), "mlp forward kernel");
}

extern "C" int pdg_mlp_backward(int max_rows, const int *d_rows, int n, int k, const float *d_dz, const void *d_w, const float *d_zin,
                                const float *d_hin, float *d_dzin, int segments, float *d_part, void *stream)
{
    if (max_rows <= 0 || !d_rows || !d_dz || !d_w || !d_hin || !d_part || segments < 1 || (d_dzin && !d_zin))
        return fail(PDG_BAD_ARGUMENT, "pdg_mlp_backward: bad argument");
    launch_mlp_backward(max_rows, d_rows, n, k, d_dz, d_w, d_zin, d_hin, d_dzin, segments, d_part, (cudaStream_t)stream);
    return cuda_check(cudaGetLastError(), "mlp backward kernels");
}

extern "C" int pdg_mlp_adam(int n, int k, int segments, const float *d_part, float scale, float *d_wm, float *d_bm, float *d_m1, float *d_m2,
                            void *d_w, float lr, float beta1, float beta2, int step, void *stream)
{
    if (!d_part || !d_wm || !d_bm || !d_m1 || !d_m2 || !d_w || step < 1) return fail(PDG_BAD_ARGUMENT, "pdg_mlp_adam: bad argument");
    const float c1 = 1.0f / (1.0f - powf(beta1, (float)step)), c2 = 1.0f / (1.0f - powf(beta2, (float)step));
    launch_mlp_adam(n, k, segments, d_part, scale, d_wm, d_bm, d_m1, d_m2, d_w, lr, beta1, beta2, c1, c2, (cudaStream_t)stream);
    return cuda_check(cudaGetLastError(), "mlp adam kernel");
}

extern "C" int pdg_guess_assemble(pdg_system *s, int n_frames, const double *d_xyz, const int *d_offsets, const int *d_row_pair,
                                  const float *d_y, double *d_density, void *stream)
{
    if (!s || n_frames <= 0 || !d_xyz || !d_offsets || !d_row_pair || !d_y || !d_density) return fail(PDG_BAD_ARGUMENT, "pdg_guess_assemble: bad argument");
    launch_guess_assemble(s->d, n_frames, d_xyz, d_offsets, d_row_pair, d_y, d_density, (cudaStream_t)stream);
    return cuda_check(cudaGetLastError(), "guess assembly kernel");
}

extern "C" int pdg_guess_loss(pdg_system *s, int n_frames, const double *d_xyz, const int *d_offsets, const int *d_row_pair,
                              const double *d_density, const double *d_target, float *d_dy, double *d_loss, void *stream)
{
    if (!s || n_frames <= 0 || !d_xyz || !d_offsets || !d_row_pair || !d_density || !d_target || !d_dy || !d_loss)
        return fail(PDG_BAD_ARGUMENT, "pdg_guess_loss: bad argument");
    launch_guess_loss(s->d, n_frames, d_xyz, d_offsets, d_row_pair, d_density, d_target, d_dy, d_loss, (cudaStream_t)stream);
    return cuda_check(cudaGetLastError(), "guess loss kernel");
}

// ---- Langevin dynamics and density combinations (dynamics.cu)
extern "C" int pdg_langevin_positions(int n_replicas, int n_atoms, int n_free, const int *d_free_atoms, const double *d_inv_sqrt_mass,
                                      double *d_xyz, double *d_velocities, const double *d_accelerations, const double *h_factors,
                                      int random, unsigned long long seed, unsigned int step, double *d_deviates, void *stream)
{
    if (n_replicas <= 0 || n_atoms <= 0 || n_free <= 0 || n_free > n_atoms || !d_free_atoms || !d_inv_sqrt_mass || !d_xyz ||
        !d_velocities || !d_accelerations || !h_factors)
        return fail(PDG_BAD_ARGUMENT, "pdg_langevin_positions: bad argument");
    LangevinFactors f;
    f.facR1 = h_factors[0]; f.facR2 = h_factors[1]; f.facV1 = h_factors[2]; f.facV2 = h_factors[3];
    f.sdR = h_factors[4]; f.sdV1 = h_factors[5]; f.sdV2 = h_factors[6];
    if (random < 0 || random > 2 || (random == 2 && !d_deviates)) return fail(PDG_BAD_ARGUMENT, "pdg_langevin_positions: bad random mode");
    f.random = random;
    launch_langevin_positions(n_replicas, n_atoms, n_free, d_free_atoms, d_inv_sqrt_mass, d_xyz, d_velocities, d_accelerations, f,
                              (uint64_t)seed, (uint32_t)step, d_deviates, (cudaStream_t)stream);
    return cuda_check(cudaGetLastError(), "langevin positions kernel");
}

extern "C" int pdg_langevin_velocities(int n_replicas, int n_free, int n_rows, const int *d_grad_rows, const double *d_mass,
                                       const double *d_grad_a, const double *d_grad_b, double grad_scale, double facV3,
                                       double *d_velocities, double *d_accelerations, double *d_mv2, void *stream)
{
    if (n_replicas <= 0 || n_free <= 0 || n_rows <= 0 || !d_grad_rows || !d_mass || !d_grad_a || !d_velocities || !d_accelerations)
        return fail(PDG_BAD_ARGUMENT, "pdg_langevin_velocities: bad argument");
    launch_langevin_velocities(n_replicas, n_free, n_rows, d_grad_rows, d_mass, d_grad_a, d_grad_b, grad_scale, facV3, d_velocities,
                               d_accelerations, d_mv2, (cudaStream_t)stream);
    return cuda_check(cudaGetLastError(), "langevin velocities kernel");
}

extern "C" int pdg_linear_constraints_project(int n_replicas, int n_free, int n_rows, const int *d_rows, int n_vectors,
                                              const double *d_vectors, const double *d_scale, int width, double *d_array, void *stream)
{
    if (n_replicas <= 0 || n_free <= 0 || n_rows < n_free || n_vectors < 1 || n_vectors > 6 || !d_vectors ||
        width < 1 || width > 2 || !d_array || (!d_rows && n_rows != n_free))
        return fail(PDG_BAD_ARGUMENT, "pdg_linear_constraints_project: bad argument");
    launch_linear_project(n_replicas, n_free, n_rows, d_rows, n_vectors, d_vectors, d_scale, width, d_array, (cudaStream_t)stream);
    return cuda_check(cudaGetLastError(), "linear constraints kernel");
}

extern "C" int pdg_normal_deviates(long long n_pairs, unsigned long long seed, unsigned int step, unsigned int stream_id, double *d_out,
                                   void *stream)
{
    if (n_pairs <= 0 || !d_out) return fail(PDG_BAD_ARGUMENT, "pdg_normal_deviates: bad argument");
    launch_normal_deviates(n_pairs, (uint64_t)seed, (uint32_t)step, (uint32_t)stream_id, d_out, (cudaStream_t)stream);
    return cuda_check(cudaGetLastError(), "normal deviates kernel");
}

extern "C" int pdg_density_combine(long long n, int count, const double *const *h_terms, const double *h_coefficients, double *d_out,
                                   void *stream)
{
    if (n <= 0 || count < 1 || count > PDG_MAX_DENSITY_TERMS || !h_terms || !h_coefficients || !d_out)
        return fail(PDG_BAD_ARGUMENT, "pdg_density_combine: bad argument");
    DensityTerms t;
    t.count = count;
    if (reinterpret_cast<uintptr_t>(d_out) % 16) return fail(PDG_BAD_ARGUMENT, "pdg_density_combine: output not 16-byte aligned");
    for (int k = 0; k < count; k++) {
        if (!h_terms[k] || reinterpret_cast<uintptr_t>(h_terms[k]) % 16)
            return fail(PDG_BAD_ARGUMENT, "pdg_density_combine: term missing or not 16-byte aligned");
        t.d[k] = h_terms[k];
        t.c[k] = h_coefficients[k];
    }
    launch_density_combine(n, t, d_out, (cudaStream_t)stream);
    return cuda_check(cudaGetLastError(), "density combination kernel");
}

// ---- MM/MM and QC/MM Lennard-Jones energies ----
struct pdg_mm_system {
    MMDevice d;
    double *d_real = nullptr;   // charges, then the four LJ tables
    int *d_int = nullptr;       // LJ types, exclusion offsets and partners, 1-4 offsets and partners
    unsigned char *d_flags = nullptr;
};

// PairwiseInteractionABFS_MakeFactors (PairwiseInteraction.c:89-140) for the MM/MM interaction.
static MMFactors mm_factors(double inner, double outer, double damp)
{
    MMFactors f;
    f.r2Damp = damp * damp; f.r2Off = outer * outer; f.r2On = inner * inner;
    const double gamma = std::pow(f.r2Off - f.r2On, 3);
    f.a = f.r2Off * f.r2Off * (f.r2Off - 3.0 * f.r2On) / gamma;
    f.b = 6.0 * f.r2Off * f.r2On / gamma;
    f.c = -(f.r2Off + f.r2On) / gamma;
    f.d = 0.4 / gamma;
    f.qShift1 = 8.0 * (f.r2Off * f.r2On * (outer - inner) - 0.2 * (outer * f.r2Off * f.r2Off - inner * f.r2On * f.r2On)) / gamma;
    f.qShift2 = -(f.a / outer) + f.b * outer + f.c * outer * f.r2Off + f.d * outer * f.r2Off * f.r2Off;
    f.qF0 = f.qAlpha = f.aF0 = f.aAlpha = f.bF0 = f.bAlpha = 0.0;
    if (damp > 0.0) {
        const double g = -1.0 / f.r2Damp, fq = 1.0 / damp + f.qShift1;
        f.qF0 = fq - 0.5 * damp * g; f.qAlpha = -0.5 * g / damp;
    }
    f.aF6 = 1.0 / (f.r2Off * f.r2Off * f.r2Off);
    f.aK12 = std::pow(f.r2Off, 3) / (std::pow(f.r2Off, 3) - std::pow(f.r2On, 3));
    f.aShift12 = 1.0 / std::pow(inner * outer, 6);
    f.bF3 = 1.0 / (outer * f.r2Off);
    f.bK6 = (outer * f.r2Off) / (outer * f.r2Off - inner * f.r2On);
    f.bShift6 = 1.0 / std::pow(inner * outer, 3);
    if (damp > 0.0) {
        const double s12 = 1.0 / std::pow(damp, 12), fa = s12 - f.aShift12, ga = -12.0 * s12 / damp;
        f.aF0 = fa - 0.5 * damp * ga; f.aAlpha = -0.5 * ga / damp;
        const double s6 = 1.0 / std::pow(damp, 6), fb = -s6 + f.bShift6, gb = 6.0 * s6 / damp;
        f.bF0 = fb - 0.5 * damp * gb; f.bAlpha = -0.5 * gb / damp;
    }
    return f;
}

// pair list (i, j) -> offsets (n + 1) and partners, both directions, partners in list order
static void mm_csr(int n, int np, const int *pairs, std::vector<int> &start, std::vector<int> &idx)
{
    start.assign((size_t)n + 1, 0);
    for (int k = 0; k < np; k++) { start[pairs[2 * k] + 1]++; start[pairs[2 * k + 1] + 1]++; }
    for (int i = 0; i < n; i++) start[i + 1] += start[i];
    idx.assign((size_t)start[n], 0);
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int k = 0; k < np; k++) {
        const int i = pairs[2 * k], j = pairs[2 * k + 1];
        idx[fill[i]++] = j; idx[fill[j]++] = i;
    }
}

extern "C" int pdg_mm_create(int n_atoms, const double *h_charges, const int *h_lj_types, const unsigned char *h_flags, int n_lj_types,
                             const double *h_table_a, const double *h_table_b, const double *h_table_a14, const double *h_table_b14,
                             int n_exclusions, const int *h_exclusions, int n_pairs14, const int *h_pairs14, double inner_cutoff,
                             double outer_cutoff, double damping_cutoff, double dielectric, double electrostatic_scale14,
                             pdg_mm_system **out)
{
    if (!out || n_atoms <= 0 || !h_charges || !h_lj_types || !h_flags || n_lj_types <= 0 || !h_table_a || !h_table_b ||
        !h_table_a14 || !h_table_b14 || n_exclusions < 0 || n_pairs14 < 0 || (n_exclusions > 0 && !h_exclusions) ||
        (n_pairs14 > 0 && !h_pairs14))
        return fail(PDG_BAD_ARGUMENT, "pdg_mm_create: bad argument");
    if (!(damping_cutoff >= 0.0 && damping_cutoff < inner_cutoff && inner_cutoff < outer_cutoff && dielectric > 0.0))
        return fail(PDG_BAD_ARGUMENT, "pdg_mm_create: cutoffs must satisfy 0 <= damping < inner < outer, dielectric > 0");
    for (int i = 0; i < n_atoms; i++) {
        if (h_lj_types[i] < 0 || h_lj_types[i] >= n_lj_types) return fail(PDG_BAD_ARGUMENT, "pdg_mm_create: LJ type out of range");
        if (h_flags[i] & ~7) return fail(PDG_BAD_ARGUMENT, "pdg_mm_create: unknown atom flag");
        if ((h_flags[i] & MM_FLAG_MM) && (h_flags[i] & MM_FLAG_QC_LJ))
            return fail(PDG_BAD_ARGUMENT, "pdg_mm_create: an atom is either an MM atom or a QC atom");
    }
    for (int k = 0; k < n_exclusions + n_pairs14; k++) {
        const int *p = k < n_exclusions ? h_exclusions + 2 * k : h_pairs14 + 2 * (k - n_exclusions);
        if (p[0] < 0 || p[0] >= n_atoms || p[1] < 0 || p[1] >= n_atoms || p[0] == p[1])
            return fail(PDG_BAD_ARGUMENT, "pdg_mm_create: pair index out of range or self pair");
    }
    std::vector<int> es, ei, ps, pi;
    mm_csr(n_atoms, n_exclusions, h_exclusions, es, ei);
    mm_csr(n_atoms, n_pairs14, h_pairs14, ps, pi);
    const size_t nt2 = (size_t)n_lj_types * n_lj_types;
    std::vector<double> real((size_t)n_atoms + 4 * nt2);
    std::copy(h_charges, h_charges + n_atoms, real.begin());
    std::copy(h_table_a, h_table_a + nt2, real.begin() + n_atoms);
    std::copy(h_table_b, h_table_b + nt2, real.begin() + n_atoms + nt2);
    std::copy(h_table_a14, h_table_a14 + nt2, real.begin() + n_atoms + 2 * nt2);
    std::copy(h_table_b14, h_table_b14 + nt2, real.begin() + n_atoms + 3 * nt2);
    std::vector<int> ints;
    ints.insert(ints.end(), h_lj_types, h_lj_types + n_atoms);
    const size_t o_es = ints.size(); ints.insert(ints.end(), es.begin(), es.end());
    const size_t o_ei = ints.size(); ints.insert(ints.end(), ei.begin(), ei.end());
    const size_t o_ps = ints.size(); ints.insert(ints.end(), ps.begin(), ps.end());
    const size_t o_pi = ints.size(); ints.insert(ints.end(), pi.begin(), pi.end());
    ints.push_back(0);   // never an empty allocation
    pdg_mm_system *m = new pdg_mm_system();
    int rc;
    if ((rc = cuda_check(cudaMalloc(&m->d_real, sizeof(double) * real.size()), "allocate MM tables")) ||
        (rc = cuda_check(cudaMalloc(&m->d_int, sizeof(int) * ints.size()), "allocate MM lists")) ||
        (rc = cuda_check(cudaMalloc(&m->d_flags, (size_t)n_atoms), "allocate MM flags")) ||
        (rc = cuda_check(cudaMemcpy(m->d_real, real.data(), sizeof(double) * real.size(), cudaMemcpyHostToDevice), "copy MM tables")) ||
        (rc = cuda_check(cudaMemcpy(m->d_int, ints.data(), sizeof(int) * ints.size(), cudaMemcpyHostToDevice), "copy MM lists")) ||
        (rc = cuda_check(cudaMemcpy(m->d_flags, h_flags, (size_t)n_atoms, cudaMemcpyHostToDevice), "copy MM flags"))) {
        pdg_mm_destroy(m);
        return rc;
    }
    MMDevice &d = m->d;
    d.n_atoms = n_atoms; d.n_types = n_lj_types;
    d.charge = m->d_real;
    d.A = m->d_real + n_atoms; d.B = d.A + nt2; d.A14 = d.B + nt2; d.B14 = d.A14 + nt2;
    d.lj_type = m->d_int;
    d.excl_start = m->d_int + o_es; d.excl = m->d_int + o_ei; d.p14_start = m->d_int + o_ps; d.p14 = m->d_int + o_pi;
    d.flags = m->d_flags;
    d.fac = mm_factors(inner_cutoff, outer_cutoff, damping_cutoff);
    // UNITS_ENERGY_E2ANGSTROMS_TO_KILOJOULES_PER_MOLE (pCore-1.9.0/extensions/cinclude/Units.h:18-49)
    const double e2a_kj = (1.0e7 * 6.0221415e23 * 1.60217653e-19 * 1.60217653e-19) / (4.0 * M_PI * 8.854187817e-12);
    d.escale = e2a_kj / dielectric;
    d.escale14 = d.escale * electrostatic_scale14;
    d.outer = outer_cutoff;
    *out = m;
    return PDG_OK;
}

extern "C" int pdg_mm_destroy(pdg_mm_system *m)
{
    if (!m) return PDG_OK;
    if (m->d_real) cudaFree(m->d_real);
    if (m->d_int) cudaFree(m->d_int);
    if (m->d_flags) cudaFree(m->d_flags);
    delete m;
    return PDG_OK;
}

extern "C" size_t pdg_mm_workspace_bytes(const pdg_mm_system *m, int n_frames)
{
    if (!m || n_frames <= 0) return 0;
    return mm_layout(m->d.n_atoms).stride * (size_t)n_frames;
}

extern "C" int pdg_mm_energy_gradients(const pdg_mm_system *m, int n_frames, const double *d_xyz, double *d_energies, double *d_gradients,
                                       void *d_workspace, size_t workspace_bytes, void *stream)
{
    if (!m || n_frames <= 0 || n_frames > 65535 || !d_xyz || !d_energies || !d_workspace)
        return fail(PDG_BAD_ARGUMENT, "pdg_mm_energy_gradients: bad argument");
    if (workspace_bytes < pdg_mm_workspace_bytes(m, n_frames)) return fail(PDG_BAD_ARGUMENT, "pdg_mm_energy_gradients: workspace too small");
    if (reinterpret_cast<uintptr_t>(d_workspace) % 256) return fail(PDG_BAD_ARGUMENT, "pdg_mm_energy_gradients: workspace not 256-byte aligned");
    launch_mm_energy(m->d, n_frames, d_xyz, d_energies, d_gradients, (char *)d_workspace, (cudaStream_t)stream);
    return cuda_check(cudaGetLastError(), "MM/MM energy kernels");
}
