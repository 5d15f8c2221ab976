// Monte Carlo pivot and jump moves over a batch (src/monte_carlo_sampler.cpp).
// Every system of the batch takes its step at once: one energy evaluation of
// the batch before and one after the proposals, which one kernel makes for
// all systems (a block per system); the Metropolis tests run on the host.
#include <cmath>
#include <cstring>

#include "dev_math.cuh"
#include "launch.cuh"
#include "mc.h"

namespace ug {

namespace {

// rotation by `angle` about the unit vector `a` (axis_angle_to_rot,
// src/affine.h:49-64), row-major
__device__ void axis_angle(float* U, float angle, f3 a) {
    float c = cosf(angle), s = sinf(angle), C = 1.f - c;
    U[0] = a.x * a.x * C + c;       U[1] = a.x * a.y * C - a.z * s; U[2] = a.x * a.z * C + a.y * s;
    U[3] = a.y * a.x * C + a.z * s; U[4] = a.y * a.y * C + c;       U[5] = a.y * a.z * C - a.x * s;
    U[6] = a.z * a.x * C - a.y * s; U[7] = a.z * a.y * C + a.x * s; U[8] = a.z * a.z * C + c;
}
__device__ __forceinline__ f3 unit(f3 v) { return v * (1.f / sqrtf(mag2(v))); }
// dihedral angle in [-pi, pi] of four points (the reference's dihedral_germ
// convention, src/vector_math.h:766-798)
__device__ float dihedral(f3 r1, f3 r2, f3 r3, f3 r4) {
    f3 F = r1 - r2, G = r2 - r3, H = r4 - r3;
    f3 A = cross(F, G), B = cross(H, G), C = cross(B, A);
    return atan2f(dot(C, G), dot(A, B) * sqrtf(mag2(G)));
}

// Pivot proposal (PivotSampler::propose_random_move,
// src/monte_carlo_sampler.cpp:84-155): a location and a (phi, psi) bin drawn
// from the location's proposal table, a point inside the bin; the C-terminal
// side is rotated about CA-N by the change of phi and about C-CA by the
// change of psi.
__global__ void mc_pivot_kernel(McDev m, float* pos, unsigned long long round) {
    grid_dep_entry();
    const int s = blockIdx.x;
    const int l0 = m.piv_off[s], nloc = m.piv_off[s + 1] - l0;
    if (nloc == 0) return;  // block-uniform
    __shared__ float U1[9], U2[9], o1[3], o2[3];
    __shared__ int mv[4];
    if (threadIdx.x == 0) {
        const float PIf = 3.14159265358979f;
        uint32_t key[4] = {m.seed[s], 2u, 0u, 0u};  // PIVOT_MOVE_RANDOM_STREAM
        uint32_t ctr[4] = {uint32_t(round & 0xffffffffu), uint32_t(round >> 32), 0u, 0u};
        uint32_t b[4];
        threefry4x32(ctr, key, b);
        ctr[3]++;
        float ux = u01f(b[0]), uy = u01f(b[1]), uz = u01f(b[2]), uw = u01f(b[3]);
        int loc = int(float(nloc) * uz);
        if (loc == nloc) loc--;
        loc += l0;
        const int nb = m.n_bin[s], nbb = nb * nb;
        const size_t t0 = size_t(m.tab_off[s]) + size_t(m.piv_layer[loc]) * size_t(nbb);
        const float* cdf = m.prop_cdf + t0;
        const float* pot = m.prop_pot + t0;
        int a = 0, z = nbb;  // first bin whose cumulative probability is >= uw
        while (a < z) {
            int mid = (a + z) >> 1;
            if (cdf[mid] < uw) a = mid + 1;
            else z = mid;
        }
        if (a >= nbb) a = nbb - 1;
        const float new_lp = pot[a];
        const int phi_bin = a / nb, psi_bin = a % nb;
        const float w = 2.f * PIf / float(nb);
        const float nphi = w * (float(phi_bin) + ux - 0.5f) - PIf;
        const float npsi = w * (float(psi_bin) + uy - 0.5f) - PIf;
        const int* at = m.piv_atom + 5 * size_t(loc);
        f3 prevC = ld3(pos + 3 * size_t(at[0])), N = ld3(pos + 3 * size_t(at[1])), CA = ld3(pos + 3 * size_t(at[2])),
           C = ld3(pos + 3 * size_t(at[3])), nN = ld3(pos + 3 * size_t(at[4]));
        const float ophi = dihedral(prevC, N, CA, C), opsi = dihedral(N, CA, C, nN);
        int obp = int((ophi + PIf) * (0.5f / PIf) * float(nb) + 0.5f);  // undo the half-bin shift
        int obs = int((opsi + PIf) * (0.5f / PIf) * float(nb) + 0.5f);
        obp = obp >= nb ? 0 : obp;
        obs = obs >= nb ? 0 : obs;
        const float old_lp = pot[obp * nb + obs];
        axis_angle(U1, nphi - ophi, unit(CA - N));
        axis_angle(U2, npsi - opsi, unit(C - CA));
        o1[0] = CA.x; o1[1] = CA.y; o1[2] = CA.z;
        o2[0] = C.x; o2[1] = C.y; o2[2] = C.z;
        mv[0] = at[3];
        mv[1] = at[4];
        mv[2] = m.piv_range[2 * loc];
        mv[3] = m.piv_range[2 * loc + 1];
        m.delta_lprob[s] = new_lp - old_lp;
        threefry4x32(ctr, key, b);
        m.u_accept[s] = u01f(b[0]);
    }
    __syncthreads();
    const f3 O1 = mk(o1[0], o1[1], o1[2]), O2 = mk(o2[0], o2[1], o2[2]);
    const int n_mv = 2 + max(0, mv[3] - mv[2]);
    for (int i = threadIdx.x; i < n_mv; i += blockDim.x) {
        int a = i == 0 ? mv[0] : i == 1 ? mv[1] : mv[2] + i - 2;
        f3 y = ld3(pos + 3 * size_t(a));
        f3 t = O2 + rot(U2, y - O2);
        st3(pos + 3 * size_t(a), O1 + rot(U1, t - O1));
    }
}

// Jump proposal (JumpSampler::propose_random_move,
// src/monte_carlo_sampler.cpp:200-245): a random chain is translated by a
// Gaussian displacement or rotated about its centroid by a Gaussian angle
// about a random axis.
__global__ void mc_jump_kernel(McDev m, float* pos, unsigned long long round) {
    grid_dep_entry();
    const int s = blockIdx.x;
    const int c0 = m.jmp_off[s], nch = m.jmp_off[s + 1] - c0;
    if (nch == 0) return;  // block-uniform
    __shared__ int type, first, end;
    __shared__ float U[9], disp[3];
    __shared__ float red[3][32];
    if (threadIdx.x == 0) {
        uint32_t key[4] = {m.seed[s], 3u, 0u, 0u};  // JUMP_MOVE_RANDOM_STREAM
        uint32_t ctr[4] = {uint32_t(round & 0xffffffffu), uint32_t(round >> 32), 0u, 0u};
        uint32_t b[4];
        threefry4x32(ctr, key, b);
        ctr[3]++;
        type = int(2.f * u01f(b[0]));
        int ch = int(float(nch) * u01f(b[3]));
        if (ch == nch) ch--;
        ch += c0;
        first = m.jmp_range[2 * ch];
        end = m.jmp_range[2 * ch + 1];
        threefry4x32(ctr, key, b);
        ctr[3]++;
        float n0, n1, n2, n3;
        box_muller(b[0], b[1], n0, n1);
        box_muller(b[2], b[3], n2, n3);
        if (type == 0) {
            float sc = m.jmp_trans[ch] / sqrtf(3.f);
            disp[0] = sc * n0;
            disp[1] = sc * n1;
            disp[2] = sc * n2;
        } else {
            f3 ax = mk(n1, n2, n3);
            ax = ax * (1.f / (sqrtf(mag2(ax)) + 1e-16f));
            axis_angle(U, m.jmp_rot[ch] * n0, ax);
        }
        m.delta_lprob[s] = m.prob_mod[s];
        threefry4x32(ctr, key, b);
        m.u_accept[s] = u01f(b[0]);
    }
    __syncthreads();
    if (type == 0) {
        for (int a = first + int(threadIdx.x); a < end; a += blockDim.x) {
            pos[3 * size_t(a)] += disp[0];
            pos[3 * size_t(a) + 1] += disp[1];
            pos[3 * size_t(a) + 2] += disp[2];
        }
        return;
    }
    // centroid of the chain, then the rotation about it
    f3 c = mk(0.f, 0.f, 0.f);
    for (int a = first + int(threadIdx.x); a < end; a += blockDim.x) c += ld3(pos + 3 * size_t(a));
    for (int o = 16; o > 0; o >>= 1) {
        c.x += __shfl_xor_sync(0xffffffffu, c.x, o);
        c.y += __shfl_xor_sync(0xffffffffu, c.y, o);
        c.z += __shfl_xor_sync(0xffffffffu, c.z, o);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) {
        red[0][warp] = c.x;
        red[1][warp] = c.y;
        red[2][warp] = c.z;
    }
    __syncthreads();
    f3 com = mk(0.f, 0.f, 0.f);
    for (int w = 0; w < nw; ++w) com += mk(red[0][w], red[1][w], red[2][w]);
    com = com * (1.f / float(end - first));
    for (int a = first + int(threadIdx.x); a < end; a += blockDim.x) {
        f3 y = ld3(pos + 3 * size_t(a));
        st3(pos + 3 * size_t(a), com + rot(U, y - com));
    }
}

std::vector<float> read_f32(h5lite::File& f, const std::string& p) { return f.read<float>(p); }
std::vector<int> read_i32(h5lite::File& f, const std::string& p) { return f.read<int32_t>(p); }

}  // namespace

McSampler::McSampler(Engine& e, const std::vector<std::string>& paths) : e_(e) {
    const int S = e.n_sys;
    if (int(paths.size()) != S) throw Error("Monte Carlo sampler: one configuration per system");
    has_pivot.assign(size_t(S), 0);
    has_jump.assign(size_t(S), 0);
    std::vector<int> piv_off{0}, piv_atom, piv_range, piv_layer, tab_off, n_bin, jmp_off{0}, jmp_range;
    std::vector<float> pot_all, cdf_all, jmp_trans, jmp_rot, prob_mod;
    for (int s = 0; s < S; ++s) {
        h5lite::File f(paths[size_t(s)]);
        const int a0 = e.atom_off[size_t(s)], na = e.n_atom[size_t(s)];
        tab_off.push_back(int(pot_all.size()));
        int nb = 0;
        if (f.exists("/input/pivot_moves")) {
            const std::string g = "/input/pivot_moves/";
            auto d = f.dims(g + "proposal_pot");
            if (d.size() != 3 || d[1] != d[2]) throw Error("pivot_moves/proposal_pot must be (layers, bins, bins)");
            const int nl = int(d[0]);
            nb = int(d[1]);
            auto pa = read_i32(f, g + "pivot_atom");
            auto pr = read_i32(f, g + "pivot_range");
            auto rt = read_i32(f, g + "pivot_restype");
            const size_t nloc = rt.size();
            if (pa.size() != 5 * nloc || pr.size() != 2 * nloc) throw Error("pivot_moves arrays have different lengths");
            for (size_t l = 0; l < nloc; ++l) {
                if (rt[l] < 0 || rt[l] >= nl) throw Error("invalid pivot restype");
                for (int k = 0; k < 5; ++k) {
                    int x = pa[5 * l + size_t(k)];
                    if (x < 0 || x >= na) throw Error("pivot_atom out of range");
                    if (pr[2 * l] <= x && x < pr[2 * l + 1])
                        throw Error("pivot_range cannot contain any atoms in pivot_atom");
                    piv_atom.push_back(a0 + x);
                }
                if (pr[2 * l] < 0 || pr[2 * l + 1] > na || pr[2 * l] > pr[2 * l + 1])
                    throw Error("pivot_range out of range");
                piv_range.push_back(a0 + pr[2 * l]);
                piv_range.push_back(a0 + pr[2 * l + 1]);
                piv_layer.push_back(rt[l]);
            }
            // normalised -log probability and cumulative probability per layer
            // (src/monte_carlo_sampler.cpp:60-78: sums in double, stored in float)
            auto pp = read_f32(f, g + "proposal_pot");
            const size_t nbb = size_t(nb) * size_t(nb);
            std::vector<float> cdf(pp.size());
            for (int layer = 0; layer < nl; ++layer) {
                double sum = 0.;
                for (size_t i = 0; i < nbb; ++i) {
                    sum += std::exp(-double(pp[size_t(layer) * nbb + i]));
                    cdf[size_t(layer) * nbb + i] = float(sum);
                }
                double inv = 1. / sum, lsum = std::log(sum);
                for (size_t i = 0; i < nbb; ++i) {
                    size_t k = size_t(layer) * nbb + i;
                    cdf[k] = float(double(cdf[k]) * inv);
                    pp[k] = float(double(pp[k]) + lsum);
                }
                cdf[(size_t(layer) + 1) * nbb - 1] = 1.f;
            }
            pot_all.insert(pot_all.end(), pp.begin(), pp.end());
            cdf_all.insert(cdf_all.end(), cdf.begin(), cdf.end());
            has_pivot[size_t(s)] = nloc > 0;
            any_pivot = any_pivot || nloc > 0;
        }
        n_bin.push_back(nb);
        piv_off.push_back(int(piv_layer.size()));
        float pm = 0.f;
        if (f.exists("/input/jump_moves")) {
            const std::string g = "/input/jump_moves/";
            auto ar = read_i32(f, g + "atom_range");
            auto st = read_f32(f, g + "sigma_trans");
            auto sr = read_f32(f, g + "sigma_rot");
            if (ar.size() != 2 * st.size() || st.size() != sr.size()) throw Error("jump_moves arrays have different lengths");
            for (size_t c = 0; c < st.size(); ++c) {
                if (ar[2 * c] < 0 || ar[2 * c + 1] > na || ar[2 * c] >= ar[2 * c + 1]) throw Error("jump atom_range out of range");
                jmp_range.push_back(a0 + ar[2 * c]);
                jmp_range.push_back(a0 + ar[2 * c + 1]);
                jmp_trans.push_back(st[c]);
                jmp_rot.push_back(sr[c]);
            }
            if (f.has_attr("/input/jump_moves", "prob_mod"))
                pm = f.attr_values<float>("/input/jump_moves", "prob_mod").at(0);
            has_jump[size_t(s)] = !st.empty();
            any_jump = any_jump || !st.empty();
        }
        prob_mod.push_back(pm);
        jmp_off.push_back(int(jmp_trans.size()));
    }
    auto up_i = [&](const std::vector<int>& v) { return e.upload(v.empty() ? std::vector<int>{0} : v); };
    auto up_f = [&](const std::vector<float>& v) { return e.upload(v.empty() ? std::vector<float>{0.f} : v); };
    d_.n_sys = S;
    d_.seed = e.d_seed;
    d_.piv_off = up_i(piv_off);
    d_.piv_atom = up_i(piv_atom);
    d_.piv_range = up_i(piv_range);
    d_.piv_layer = up_i(piv_layer);
    d_.tab_off = up_i(tab_off);
    d_.n_bin = up_i(n_bin);
    d_.prop_pot = up_f(pot_all);
    d_.prop_cdf = up_f(cdf_all);
    d_.jmp_off = up_i(jmp_off);
    d_.jmp_range = up_i(jmp_range);
    d_.jmp_trans = up_f(jmp_trans);
    d_.jmp_rot = up_f(jmp_rot);
    d_.prob_mod = up_f(prob_mod);
    d_.delta_lprob = e.alloc<float>(size_t(S));
    d_.u_accept = e.alloc<float>(size_t(S));
    saved_ = e.alloc<float>(3 * size_t(e.atom_total));
    for (auto& v : success) v.assign(size_t(S), 0ull);
    for (auto& v : attempt) v.assign(size_t(S), 0ull);
}

void McSampler::step(uint64_t round, int* accepted) {
    Engine& e = e_;
    const int S = e.n_sys;
    if (accepted)
        for (int i = 0; i < 2 * S; ++i) accepted[i] = -1;
    std::vector<float> temp(static_cast<size_t>(S));
    UG_CK(cudaMemcpyAsync(temp.data(), e.d_temp, 4 * size_t(S), cudaMemcpyDeviceToHost, e.st));
    e.sync();
    const size_t pos_bytes = sizeof(float) * 3 * size_t(e.atom_total);
    for (int k = 0; k < 2; ++k) {  // the pivot sampler, then the jump sampler
        if (k == 0 ? !any_pivot : !any_jump) continue;
        const std::vector<char>& has = k == 0 ? has_pivot : has_jump;
        std::vector<double> e_old(static_cast<size_t>(S)), e_new(static_cast<size_t>(S));
        e.compute_checked(true);
        e.energies(e_old.data());
        UG_CK(cudaMemcpyAsync(saved_, e.d_pos, pos_bytes, cudaMemcpyDeviceToDevice, e.st));
        if (k == 0) ug::launch(mc_pivot_kernel, S, 128, 0, e.st, d_, e.d_pos, (unsigned long long)round);
        else ug::launch(mc_jump_kernel, S, 256, 0, e.st, d_, e.d_pos, (unsigned long long)round);
        UG_CK(cudaGetLastError());
        e.compute_checked(true);
        e.energies(e_new.data());
        std::vector<float> dl(static_cast<size_t>(S)), ua(static_cast<size_t>(S));
        UG_CK(cudaMemcpyAsync(dl.data(), d_.delta_lprob, 4 * size_t(S), cudaMemcpyDeviceToHost, e.st));
        UG_CK(cudaMemcpyAsync(ua.data(), d_.u_accept, 4 * size_t(S), cudaMemcpyDeviceToHost, e.st));
        e.sync();
        for (int s = 0; s < S; ++s) {
            if (!has[size_t(s)]) continue;
            // FP32 as the reference (src/monte_carlo_sampler.cpp:266-275)
            float lb = dl[size_t(s)] - (1.f / temp[size_t(s)]) * (float(e_new[size_t(s)]) - float(e_old[size_t(s)]));
            bool ok = lb >= 0.f || std::exp(lb) >= ua[size_t(s)];
            attempt[k][size_t(s)]++;
            if (ok) success[k][size_t(s)]++;
            else {
                size_t a0 = 3 * size_t(e.atom_off[size_t(s)]), n = 3 * size_t(e.n_atom[size_t(s)]);
                UG_CK(cudaMemcpyAsync(e.d_pos + a0, saved_ + a0, 4 * n, cudaMemcpyDeviceToDevice, e.st));
            }
            if (accepted) accepted[2 * s + k] = ok ? 1 : 0;
        }
        e.sync();
    }
}

}  // namespace ug
