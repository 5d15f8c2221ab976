// Plain structs shared by the host engine (engine.cu) and the sm_103a kernels
// (graph.cu, nodes.cu).  All pointers are device pointers.  Arrays are flattened over
// the batch: every system's elements are concatenated and all stored indices
// are global (already offset by the owning system's start).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ug {

// status bits written by kernels into Engine::d_status
enum StatusBits : int {
    ST_EDGE_OVERFLOW = 1,   // a pair list exceeded its capacity
    ST_BP_NOT_CONVERGED = 2,  // a BP solve hit max_iter
    ST_RES_EDGE_OVERFLOW = 4, // residue-pair edge storage exceeded
};

enum IKind : int { IK_ROTAMER = 0, IK_HBCOV = 1, IK_PHB = 2, IK_ENVCOV = 3, IK_HBENV = 4, IK_BACKBONE = 5 };
enum Excl : int { EX_ROTAMER = 0, EX_SEQ1 = 1, EX_SEQ2 = 2 };

// Pair list + per-edge values for one interaction graph over the whole batch.
struct DGraph {
    int kind, excl, symmetric;
    // periodic box edge lengths (0: open boundaries): pair distances then use
    // the minimum image (a mode of this engine only; the reference has none)
    float box[3];
    int d1, d2, n_param, n_type1, n_type2;
    float cutoff;
    // element sets (set2 == set1 when symmetric)
    int n1, n2;                 // total elements over the batch
    const int* loc1;            // element -> row in the arg node output
    const int* loc2;
    const int* type1;
    const int* type2;
    const int* id1;
    const int* id2;
    const int* sys1;            // element -> system
    const float* param;         // (n_type1*n_type2, n_param)
    int w1, w2;                 // row widths of the arg node outputs
    const float* in1;           // arg node outputs
    const float* in2;
    float* sens1;               // arg node sensitivities
    float* sens2;
    // pair search rows: one row = one block of 4 set-1 elements of one system
    int n_rows;
    const int* row_i1;          // first set-1 element of the row
    const int* row_i1_end;      // end of the system's set-1 range
    const int* row_i2;          // first candidate set-2 element
    const int* row_i2_end;      // end of the system's set-2 range
    int* row_count;
    int* row_off;               // exclusive scan of row_count (n_rows+1)
    const int* sys_first_row;   // per system: first row (n_sys+1)
    int n_sys;
    // edges
    int cap;
    int2* edges;                // (i1, i2) set indices
    int* n_edge;                // device scalar
    float* value;
    float* deriv;               // cap * (d1+d2)
    float* esens;
    int* eaux;                  // per-edge scratch (rotamer graph: the source of each edge's BP weight)
    float4* x1;                 // packed positions (xyz) of set 1 for the search
    float4* x2;
    int* status;
    // candidate cache (src/interaction_graph.h:51-258): per system, the pairs
    // within cutoff + buffer at the positions of that system's last rebuild;
    // every evaluation refines them to the cutoff.  cached == 0: full search
    // every evaluation.
    int cached;
    float buffer;               // 1 + 0.2 * cutoff (src/interaction_graph.h:396)
    float4* xc1;                // positions at each system's last rebuild
    float4* xc2;
    const int* sys2;            // set-2 element -> system
    int* sys_flag;              // per system: rebuilt in this evaluation
    int* cache_force;           // device scalar: rebuild every system next time
    int* sys_over;              // per system: its segment overflowed at the last rebuild
    int2* cache_edges;          // per-system segments of candidates
    const int* cache_off;       // segment starts (n_sys+1)
    int* cache_n;               // per system number of candidates
    int* active_off;            // per system prefix of refine tiles (n_sys+1)
    int max_tiles;              // refine tiles if every segment were full
    int* tile_count;            // max_tiles + 1
    int* tile_off;              // max_tiles + 1
    unsigned char* refine_mask; // per refine tile and thread: which of its 4 candidates are edges
    unsigned long long* rebuilds;  // running count of system cache rebuilds
    int* any_flag;              // device scalar: some system is rebuilt in this evaluation
    // coverage sums (hbond / environment coverage nodes; cov_out nullptr:
    // none): the edge evaluation adds each edge value into cov_out[row(e)],
    // and the scatter takes each edge's sensitivity from cov_sens[row(e)],
    // with row(e) = cov_by_first ? (cov_aa2 ? i1 * cov_n_aa + cov_aa2[i2] : i1)
    // : i2.  The pair search zeroes the cov_n sums first (the last column of
    // rows cov_w wide).  Protein hbonds (phb_row1 set): each edge value goes
    // into the last column of both its donor's and its acceptor's row
    // (phb_row1[i1], phb_row2[i2]), and the scatter forms the edge's
    // sensitivity from both rows' (src/hbond.cpp:357-435).
    float* cov_out;
    const float* cov_sens;
    int cov_n, cov_w, cov_by_first, cov_n_aa;
    const int* cov_aa2;
    const int* phb_row1;
    const int* phb_row2;
};

// candidates per refine tile (one 256-thread block, 4 per thread)
constexpr int CACHE_TILE = 1024;

// One system-batched rotamer belief-propagation problem.
struct DBP {
    int n_sys;
    int n_res;                  // residues over the batch
    const int* res_off;         // per system residue start (n_sys+1)
    const int* nrot;            // residue -> 1, 3 or 6
    const int* res_N;           // residue -> number of residues of its system
    const int* res_sys;         // residue -> system
    const int* res_local;       // residue -> index within its system
    const long long* slot_off;  // per system offset into the dense slot map
    int* slot;                  // dense (N_s x N_s) residue-pair map, -1 = none
    int* row_count;             // per residue number of neighbours
    int* row_ptr;               // n_res+1
    int* col;                   // entry -> neighbour residue (global)
    int* erow;                  // entry -> row residue
    int* rev;                   // entry -> reverse entry
    int4* einfo;                // entry -> (row node local index, reverse entry, column node local index, 0)
    int ent_cap;
    int* n_ent;
    float* esum;                // entry * 36: summed bead energies (row rot, col rot)
    float* P;                   // entry * 36: exp(-esum)
    float* msg;                 // 2 * ent_cap * 8
    float* emarg;               // entry * 36
    float* E1;                  // res * 8: 1-body energy per rotamer
    float* E1x;                 // res * 8: folded 1-rotamer-partner edge energies
    float* prob;                // res * 8
    float* eoff;                // res
    float* belief;              // 2 * n_res * 8
    float* marg;                // res * 8
    int* n_iter;                // per system
    float damping, tol;
    int max_iter, chunk;
    int max_res_sys;            // largest residue count of one system (shared-memory sizing)
    int variant;                // launch variant of the solve (bp_variant_desc)
    // solve's shared layout (set at launch): compact when dsm_cap > 0, with
    // nb_cap own-node belief slots and dsm_cap own-entry message slots per block
    int dsm_cap, nb_cap;
    float* nb_scratch;          // 2 * n_res * 8: own beliefs of a compact solve whose cluster does not fit
    // bead level
    int n_bead;
    const int* bead_res;        // bead -> residue (global)
    const int* bead_rot;        // bead -> rotamer
    const int* bead_loc;        // bead -> row in the bead node output
    const int* res_bead_off;    // residue -> its first bead (n_res+1) when the beads are in residue order, else null
    double* e11;                // per system sum of energies of 1-1 bead edges
    unsigned long long* bad_solves;  // per system: solves that ran into max_iter (cumulative)
    // per-node decomposition for the driver's logs (null: not computed):
    // free energy, average energy, entropy (res each), one-body energy of each
    // input (log_n1b x res), half of the 1-1 edge energies of each node (res)
    float *log_fe, *log_pot, *log_ent, *log_1b, *log_e11;
    int* status;
    // measurement: running per-system total of the solve kernel's algorithmic
    // bytes (the formula is in bp_solve_kernel), and optional host-side CUDA
    // events bracketing each solve launch (kt_ev null: no events recorded)
    unsigned long long* alg_bytes;
    // learned warm start: predicted marginals (res * 8; null = uniform start)
    // and per-system sweep statistics (4 floats per system)
    const float* warm;
    float* warm_stat;
    // sweeps a warm start must save to be used: the network's cost for the
    // learned start, less for a start that costs no kernels
    float warm_gain;
    // previous-solve start (reuse != 0): each solve leaves its final messages,
    // their columns and row offsets in the half `parity` of the prev_ arrays;
    // the next solve (other half) starts from them, matched by residue pair,
    // and from the previous marginals.  parity flips once per evaluation.
    int reuse;
    int* parity;                // device scalar
    int* prev_valid;            // 2 x n_sys
    int* prev_row_ptr;          // 2 x (n_res + 1)
    int* prev_col;              // 2 x ent_cap
    float* prev_msg;            // 2 x ent_cap x 8
    cudaEvent_t* kt_ev;
    int* kt_used;
    int kt_cap;
};

// dynamic shared memory of the BP solve for a system of n residues: both
// belief buffers (8 floats per node each) and the rotamer counts
inline size_t bp_solve_smem_bytes(int n) { return size_t(n) * (2 * 8 * sizeof(float) + sizeof(int)); }

// launch variants of the BP solve: blocks per system, lanes per node, threads per block
int bp_variant_count();
void bp_variant_desc(int i, int* cluster, int* lanes, int* threads);

// --------------------------------------------------------------- launchers --
// skip_unless: optional device flag; the scan does nothing when it reads 0
// exclusive scan by one block; skip_unless: run only if *skip_unless; cap >= 0:
// a total beyond cap sets `bit` in *status and is stored as cap
void launch_scan(const int* in, int* out, int n, int* total_out, cudaStream_t st, const int* skip_unless = nullptr,
                 int cap = -1, int* status = nullptr, int bit = ST_EDGE_OVERFLOW);
void launch_pack_positions(const DGraph& g, cudaStream_t st);
void launch_pairs(const DGraph& g, cudaStream_t st);
void launch_edge_eval(const DGraph& g, int* sys_start, int* sys_end, cudaStream_t st);
void launch_edge_scatter(const DGraph& g, cudaStream_t st);
void launch_param_deriv(const DGraph& g, float* out, cudaStream_t st);
// in: up to 4 one-body energy inputs (bead rows), in_sens their sensitivities
// warm: learned warm start (null: off); pos / atom_off feed its features
struct WarmDev;
void launch_bp_reset(DBP& b, cudaStream_t st);
void launch_rotamer_edges(DBP& b, const DGraph& g, cudaStream_t st);
void launch_bp_structure(DBP& b, const DGraph& g, cudaStream_t st);
void launch_bp(DBP& b, const DGraph& g, const float* const* in, float* const* in_sens, const int* w, int n_in,
               int prev_n_ent, int* scan_total, int want_energy, double* energy_out, const WarmDev* warm,
               const float* pos, const int* atom_off, cudaStream_t st);
// standalone pair list of one point set (pairlist.cu); row_count and row_off
// each hold ceil(n/4) ints, row_off one more
cudaError_t launch_point_pairs(const float* pos, int n, float cutoff, int* pairs, int cap, int* n_pairs,
                               int* row_count, int* row_off, cudaStream_t st);
// fixed device scratch for the no-allocation pair list: the largest point
// count it holds, and its address on the current device
int point_pairs_noalloc_max();
cudaError_t point_pairs_noalloc_scratch(int** out);

}  // namespace ug
