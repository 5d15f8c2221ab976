"""Seeded synthetic Upside `.up` configurations for the ff_2.1 force field.

This restates the hot-path writers of the reference config generator
(py/upside_config.py) without PyTables: the node graph, argument lists,
datasets and attributes match what `upside_config.py --fasta ...
--rama-library ... --rama-sheet-mixing-energy ... --hbond-energy ...
--reference-state-rama ... --rotamer-placement ... --dynamic-rotamer-1body
--rotamer-interaction ... --environment-potential ... --bb-environment-potential
...` writes for a single- or multi-chain protein.  Files are written with the
pure-Python HDF5 writer in h5lite.py.

Differences from the reference generator, all forced by the environment:
  * `parameters/common/rama.dat` (the Rama library) is absent from the
    reference checkout, so per-residue 72x72 Rama maps are seeded synthetic
    maps built from smooth Fourier modes around helix/sheet basins (the same
    bicubic evaluation path is exercised; the maps differ from the library).
  * Sequences are drawn uniformly over the 20 amino acids from the seed.

Writer citations (py/upside_config.py): random_initial_config :186-201,
construct_equilibrium_structure :160-184, write_dist_spring :453-483,
write_angle_spring :485-515, write_omega_spring1 :546-569, write_rama_map_pot
:761-846, rama_map_pot_ref :2401-2412, write_backbone_pair :998-1016,
write_infer_H_O :332-368, write_count_hbond :1018-1047, write_short_hbond
:1049-1075, write_rotamer_placement :1077-1201, write_rotamer_backbone
:1204-1300, write_rotamer :1302-1334, write_environment :1341-1426,
write_bb_environment :1428-1538, write_weighted_pos :370-377,
write_rama_coord2 :407-446, write_affine_alignment :314-330,
write_omega_spring2 :571-673 and write_rama_map_pot2 :848-993 (--trans-cis),
read_fasta :240-253 (CPR, cis proline).
"""
import os

import numpy as np

from h5lite import H5Writer

AA = ['ALA', 'ARG', 'ASN', 'ASP', 'CYS', 'GLN', 'GLU', 'GLY', 'HIS', 'ILE',
      'LEU', 'LYS', 'MET', 'PHE', 'PRO', 'SER', 'THR', 'TRP', 'TYR', 'VAL']
BACKBONE_GROUP4 = {a: 0 for a in AA}
BACKBONE_GROUP4.update({'GLY': 1, 'PRO': 2})
N_BIT_ROTAMER = 4
DEG = np.pi / 180.

_HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_PARAMS = os.path.join(_HERE, "..", "tests", "golden", "ff21_params.npz")
_PARAM_CACHE = {}


def load_params(path=None):
    """ff_2.1 arrays (sidechain/environment/hbond/bb_env/rama reference) as a dict."""
    path = os.path.abspath(path or DEFAULT_PARAMS)
    if path not in _PARAM_CACHE:
        with np.load(path) as z:
            _PARAM_CACHE[path] = {k: z[k] for k in z.files}
    return _PARAM_CACHE[path]


# ---------------------------------------------------------------- geometry --
def _tab_matrices(phi, theta, bond_length):
    cp, sp = np.cos(phi), np.sin(phi)
    ct, st = np.cos(theta), np.sin(theta)
    r = np.zeros(phi.shape + (4, 4))
    r[..., 0, 0] = -ct
    r[..., 0, 1] = -st
    r[..., 0, 3] = -bond_length * ct
    r[..., 1, 0] = cp * st
    r[..., 1, 1] = -cp * ct
    r[..., 1, 2] = -sp
    r[..., 1, 3] = bond_length * cp * st
    r[..., 2, 0] = sp * st
    r[..., 2, 1] = -sp * ct
    r[..., 2, 2] = cp
    r[..., 2, 3] = bond_length * sp * st
    r[..., 3, 3] = 1.
    return r


def chain_from_rama(rama, angles, lengths):
    """Backbone N,CA,C positions from (phi,psi,omega), bond angles and lengths
    by chaining torsion-angle-bond affine transforms."""
    n_res = rama.shape[0]
    t = np.zeros(3 * n_res)
    t[3::3] = rama[:-1, 1]
    t[4::3] = rama[:-1, 2]
    t[5::3] = rama[1:, 0]
    mats = _tab_matrices(t, angles.ravel(), lengths.ravel())
    cur = np.eye(4)
    pos = np.zeros((3 * n_res, 3))
    for i, m in enumerate(mats):
        cur = cur @ m
        pos[i] = cur[:3, 3]
    return pos


def random_initial_config(n_res, rng):
    rama = rng.random_sample((n_res, 3)) * 2 * np.pi - np.pi
    rama[:, 2] = np.pi
    angles = np.zeros_like(rama)
    lengths = np.zeros_like(rama)
    angles[:, 0] = 120.0 * DEG
    angles[:, 1] = 120.0 * DEG
    angles[:, 2] = 109.5 * DEG
    lengths[:, 0] = 1.453
    lengths[:, 1] = 1.526
    lengths[:, 2] = 1.300
    return chain_from_rama(rama, angles, lengths)


# ----------------------------------------------------------------- rama maps --
def synthetic_rama_maps(seq, rng, n=72):
    """Seeded smooth 72x72 periodic maps (one per residue type), low in the
    alpha-helix and beta-sheet basins, with per-type random low-order Fourier
    perturbations.  Returned per residue."""
    phi = np.linspace(-np.pi, np.pi, n, endpoint=False)[:, None]
    psi = np.linspace(-np.pi, np.pi, n, endpoint=False)[None, :]

    def basin(p0, s0, w):
        return w * np.exp((np.cos(phi - p0) - 1) * 2.5 + (np.cos(psi - s0) - 1) * 2.5)

    type_maps = {}
    for aa in AA:
        m = 2.0 - basin(-63 * DEG, -43 * DEG, 2.5) - basin(-120 * DEG, 130 * DEG, 2.2)
        if aa == 'GLY':
            m = m - basin(80 * DEG, 0 * DEG, 1.5)
        if aa == 'PRO':
            m = m + 3.0 * (1 + np.cos(phi + 65 * DEG)) * 0.5
        for _ in range(6):
            kx, ky = rng.randint(0, 4, size=2)
            a, b = rng.uniform(0, 2 * np.pi, size=2)
            m = m + 0.25 * rng.randn() * np.cos(kx * phi + a) * np.cos(ky * psi + b)
        type_maps[aa] = m
    if 'CPR' in seq:
        # cis proline: drawn after the standard types, so configurations
        # without CPR keep their maps
        m = 2.0 - basin(-75 * DEG, 150 * DEG, 2.5) - basin(-80 * DEG, -20 * DEG, 1.5)
        m = m + 3.0 * (1 + np.cos(phi + 70 * DEG)) * 0.5
        for _ in range(6):
            kx, ky = rng.randint(0, 4, size=2)
            a, b = rng.uniform(0, 2 * np.pi, size=2)
            m = m + 0.25 * rng.randn() * np.cos(kx * phi + a) * np.cos(ky * psi + b)
        type_maps['CPR'] = m
    maps = np.array([type_maps[s] for s in seq])
    # maps are -log of normalized probabilities over the grid, as library maps are
    maps += np.log(np.exp(-maps).sum(axis=(-2, -1), keepdims=True))
    # remove the Boltzmann-weighted average energy as py/upside_config.py:838 does
    maps -= (maps * np.exp(-maps)).sum(axis=(-2, -1), keepdims=True)
    return maps


# ----------------------------------------------------------------- writer --
class _Cfg:
    def __init__(self, seq, chain_first_residue=()):
        self.w = H5Writer()
        self.seq = np.array(seq)
        self.n_res = len(seq)
        self.n_atom = 3 * self.n_res
        self.chain_starts = np.append([0], np.asarray(chain_first_residue, dtype=int) * 3)
        self.n_chains = len(self.chain_starts)
        self.pot = "/input/potential"

    def grp(self, name, args, **attrs):
        p = "%s/%s" % (self.pot, name)
        self.w.group(p)
        self.w.set_attr(p, "arguments", np.array([a.encode() for a in args]))
        for k, v in attrs.items():
            self.w.set_attr(p, k, v)
        return p

    def ds(self, path, value):
        self.w.dataset(path, value)

    def between_chain_ok(self, ids):
        """True for rows whose atoms all lie in one chain (find_multichain_terms)."""
        ids = np.asarray(ids)
        chain = (ids[..., None] >= self.chain_starts).sum(axis=-1)
        return np.all(chain == chain[..., :1], axis=-1)


TRANS_CIS_HEADER = 'residue init_state energy k width'
FIX_ROTAMER_HEADER = 'residue restype chain resnum chi1 chi2'


def read_trans_cis(table, seq):
    """Rows (residue, init_state, energy, k, width) of a --trans-cis table:
    a path whose first line is TRANS_CIS_HEADER, or the rows themselves
    (write_omega_spring2, py/upside_config.py:571-604).  Every residue must
    be a proline (PRO or CPR)."""
    if isinstance(table, str):
        fields = [ln.split() for ln in open(table)]
        if [x.lower() for x in fields[0]] != TRANS_CIS_HEADER.split():
            raise ValueError('First line of restraint table must be "%s"' % TRANS_CIS_HEADER)
        if not all(len(f) == 5 for f in fields):
            raise ValueError('Invalid format for restraint file')
        fields = fields[1:]
    else:
        fields = list(table)
    res = np.array([int(f[0]) for f in fields], dtype=int)
    state = np.array([int(f[1]) for f in fields], dtype=int)
    energy, k, width = (np.array([float(f[i]) for f in fields]) for i in (2, 3, 4))
    for r in res:
        if not (0 <= r < len(seq)):
            raise ValueError('Double wall energy specified for residue %i (zero is first residue) but there '
                             'are only %i residues in the FASTA' % (r, len(seq)))
        if seq[r] not in ('PRO', 'CPR'):
            raise ValueError('trans-cis residue %i is %s, not a proline' % (r, seq[r]))
    if np.any(width <= 0.):
        raise ValueError('Cannot have negative width value')
    return res, state, energy, k, width


def _chi1_state(angles):
    s = np.ones(angles.shape, dtype='i')
    s[(0. * DEG <= angles) & (angles < 120. * DEG)] = 0
    s[(-120. * DEG <= angles) & (angles < 0. * DEG)] = 2
    return s


def fix_rotamer_states(table, seq, params=None):
    """{residue: rotamer state} for a --fix-rotamer table (a path whose first
    line is FIX_ROTAMER_HEADER, or its rows): GLY and ALA take state 0;
    otherwise the states of the residue type with the same chi1 class, and
    among those the first whose chi2 offset, wrapped to (-pi, pi], is
    smallest (write_rotamer_placement, py/upside_config.py:1078-1140).
    Residues with a NaN chi1 (or a NaN chi2 where chi2 decides) stay free."""
    P = load_params(params)
    if isinstance(table, str):
        fields = [x.split() for x in open(table)]
        if [x.lower() for x in fields[0]] != FIX_ROTAMER_HEADER.split():
            raise ValueError('First line of fix-rotamer table must be "%s" but is "%s" for file %s'
                             % (FIX_ROTAMER_HEADER, " ".join(fields[0]), table))
        fields = fields[1:]
    else:
        fields = list(table)
    restype_num = {a.decode(): i for i, a in enumerate(P["sc_restype_order"])}
    tab = P["sc_restype_and_chi_and_state"]
    find_restype, find_chi2, find_state = tab[:, 0].astype('i'), tab[:, 2], tab[:, 3].astype('i')
    find_chi1_state = _chi1_state(tab[:, 1])
    fix = {}
    for residue, restype, _chain, _resnum, chi1, chi2 in fields:
        r = int(residue)
        if seq[r] != (restype if restype != 'CPR' else 'PRO'):
            raise ValueError("fix-rotamer file does not match FASTA, residue %i should be %s but fix-rotamer "
                             "file has %s" % (r, seq[r], restype))
        chi1, chi2 = float(chi1) * DEG, float(chi2) * DEG
        if restype in ('GLY', 'ALA'):
            state = 0
        else:
            if np.isnan(chi1):
                continue
            ok = (find_restype == restype_num[seq[r]]) & (find_chi1_state == _chi1_state(np.array([chi1]))[0])
            cand_chi2, cand_state = find_chi2[ok], find_state[ok]
            if len(cand_state) == 1:
                state = cand_state[0]
            else:
                if np.isnan(chi2):
                    continue
                d = (cand_chi2 - chi2) % (2 * np.pi)
                d[d > np.pi] -= 2 * np.pi
                state = cand_state[np.argmin(d)]
        fix[r] = int(state)
    return fix


def write_config(path, seq, seed, chain_first_residue=(), pos=None, environment_potential_type=1,
                 damping=0.4, chain_offsets=None, params=None, bp_tol=1e-3, moves=False,
                 jump_length_scale=5., jump_rotation_scale=30., trans_cis=None, fix_rotamer=None,
                 extra_nodes=(), membrane_thickness=None, membrane_exclude_residues=(), use_curvature=False,
                 curvature_radius=200., curvature_sign=1, surface=None, surface_included_residues=(),
                 channel_membrane=False, lateral_pressure=None):
    """Write an ff_2.1 `.up` file for `seq` (list of 3-letter codes).

    chain_first_residue: residue indices (excluding 0) where new chains start.
    pos: optional (n_atom,3) initial coordinates; otherwise random_initial_config
      per chain, chains translated by `chain_offsets` (n_chains,3) if given.
    bp_tol: the rotamer BP convergence tolerance (the recipe's 1e-3).
    moves: write the Monte Carlo move tables as the reference's config script
      does (py/upside_config.py:2520-2552): jump moves of whole chains for
      several chains (widths jump_length_scale in angstrom and
      jump_rotation_scale in degrees), pivot moves otherwise.
    trans_cis: a --trans-cis table (path or rows, see read_trans_cis): the
      omega of each listed proline gets the four-segment sigmoid barrier
      (SigmoidEnergy) instead of a spring, and its Rama potential becomes the
      omega-weighted mixture of trans and cis maps (RamaMap2 over
      SigmoidCoord/Add/Multiply switches).
    fix_rotamer: a --fix-rotamer table (path or rows, see fix_rotamer_states)
      or a {residue: state} dict; fixed residues keep one rotamer.
    seq may hold CPR (cis proline): its omega spring targets 0 and it has
    its own Rama map; every other term treats it as PRO.
    extra_nodes: further nodes, each (name, arguments, attributes dict,
      datasets dict), written after the standard ones.
    membrane_thickness: write the ff_2.1 membrane potential for a bilayer of
      this thickness (angstrom) normal to z, as --membrane-potential does:
      burial- and depth-dependent CB energies, depth-dependent energies of
      free and bonded backbone H/O, a CB placement and the curvature centre
      (write_membrane_potential3, py/upside_config.py:1727-1835, and write_CB
      :379-395).  membrane_exclude_residues skip the CB term; use_curvature,
      curvature_radius and curvature_sign bend the bilayer into a sphere.
    surface: write the `surface` node with this method (0 fast, 1 lipid
      diffusion), as --surface / --surface-method do (write_surface_coord,
      py/upside_config.py:1544-1602), over surface_included_residues if
      given; needs membrane_thickness.
    channel_membrane: write the surface-dependent membrane terms
      (cb_surf_membrane_potential, hb_surf_membrane_potential with their
      inner-residue tables) in place of cb/hb_membrane_potential, as
      --channel-membrane-potential does (write_membrane_potential4,
      py/upside_config.py:1837-1953); needs surface.
    lateral_pressure: a --membrane-lateral-potential table (path or rows of
      z, pressure in bar): the membranelateral_potential node
      (write_membrane_lateral_potential, py/upside_config.py:1955-2021);
      needs surface.
    """
    P = load_params(params)
    rng = np.random.RandomState(seed)
    seq_cpr = np.array(seq)
    seq = [s if s != 'CPR' else 'PRO' for s in seq]
    tc = read_trans_cis(trans_cis, seq_cpr) if trans_cis is not None else None
    if fix_rotamer is None:
        fix = {}
    elif isinstance(fix_rotamer, dict):
        fix = {int(r): int(v) for r, v in fix_rotamer.items()}
    else:
        fix = fix_rotamer_states(fix_rotamer, seq, params)
    c = _Cfg(seq, chain_first_residue)
    n_res, n_atom = c.n_res, c.n_atom
    w = c.w

    # ---- sequence and coordinates
    w.dataset("/input/sequence", np.array([s.encode() for s in seq_cpr]))
    if pos is None:
        starts = list(np.asarray(chain_first_residue, dtype=int))
        bounds = [0] + starts + [n_res]
        pos = np.zeros((n_atom, 3))
        for ci in range(len(bounds) - 1):
            a, b = bounds[ci], bounds[ci + 1]
            p = random_initial_config(b - a, rng)
            p -= p.mean(axis=0)
            if chain_offsets is not None:
                p += chain_offsets[ci]
            pos[3 * a:3 * b] = p
    w.dataset("/input/pos", np.asarray(pos, dtype=np.float32)[:, :, None])
    if len(chain_first_residue):
        w.dataset("/input/chain_break/chain_first_residue", np.asarray(chain_first_residue, dtype=np.int32))
    w.group("/input/args")
    w.set_attr("/input/args", "generator", "upside2-md_gb300 config_gen seed=%d" % seed)
    w.group(c.pot)

    # ---- bonded springs
    ids = np.arange(n_atom - 1)
    ids = np.column_stack((ids, ids + 1))
    eq = np.zeros(ids.shape[0])
    eq[0::3], eq[1::3], eq[2::3] = 1.453, 1.526, 1.300
    keep = c.between_chain_ok(ids)
    g = c.grp("Distance3D", ["pos", "pos"])
    c.ds(g + "/id", ids[keep])
    g = c.grp("Spring_bond", ["Distance3D"], integrator_level=0, dim1=0, pbc=0, box_len=0)
    c.ds(g + "/id", np.arange(keep.sum()))
    c.ds(g + "/equil_dist", eq[keep])
    c.ds(g + "/spring_const", 48. * np.ones(keep.sum()))

    ids = np.arange(n_atom - 2)
    ids = np.column_stack((ids, ids + 2, ids + 1))
    eq = np.zeros(ids.shape[0])
    eq[0::3] = np.cos(109.5 * DEG)
    eq[1::3] = np.cos(120.0 * DEG)
    eq[2::3] = np.cos(120.0 * DEG)
    keep = c.between_chain_ok(ids)
    g = c.grp("Angle", ["pos"])
    c.ds(g + "/id", ids[keep])
    g = c.grp("Spring_angle", ["Angle"], integrator_level=0, dim1=0, pbc=0, box_len=0)
    c.ds(g + "/id", np.arange(keep.sum()))
    c.ds(g + "/equil_dist", eq[keep])
    c.ds(g + "/spring_const", 175. * np.ones(keep.sum()))

    ids = np.arange(1, n_atom - 3, 3)
    ids = np.column_stack((ids, ids + 1, ids + 2, ids + 3))
    ids = ids[c.between_chain_ok(ids)]
    rid = (ids[:, 3] - 1) // 3  # the residue the omega leads into
    target = np.where(seq_cpr[rid] == 'CPR', 0. * DEG, 180. * DEG)
    free = np.ones(len(ids), bool) if tc is None else ~np.isin(rid, tc[0])
    g = c.grp("Dihedral_omega", ["pos"])
    c.ds(g + "/id", ids[free])
    g = c.grp("Spring_omega", ["Dihedral_omega"], integrator_level=0, dim1=0, pbc=1, box_len=np.pi * 2)
    c.ds(g + "/id", np.arange(free.sum()))
    c.ds(g + "/equil_dist", target[free])
    c.ds(g + "/spring_const", 30. * np.ones(free.sum()))
    if tc is not None:
        # double-well barrier on the trans-cis omegas: four compact-sigmoid
        # segments over [-pi, pi] (write_omega_spring2)
        res_tc, _, energy, kk, width = tc
        n_pro = len(res_tc)
        g = c.grp("Dihedral_OmegaTransCis", ["pos"])
        c.ds(g + "/id", ids[~free])
        one, sharp = np.ones(n_pro), 1. / (width * DEG)
        border = np.linspace(-np.pi, np.pi, 9)
        seg_a = [energy, energy * (1. - kk), energy, energy * 0.]
        seg_b = [-energy, energy * kk, -energy * kk, energy]
        for si, nm in enumerate(['trans1', 'cis0', 'cis1', 'trans0']):
            g = c.grp("SigmoidEnergy_" + nm, ["Dihedral_OmegaTransCis"], integrator_level=0, use_cutoff=1, dim1=0)
            c.ds(g + "/id", np.arange(n_pro))
            c.ds(g + "/a", seg_a[si])
            c.ds(g + "/b", seg_b[si])
            c.ds(g + "/c", one * border[2 * si + 1])
            c.ds(g + "/s", sharp)
            c.ds(g + "/min", one * border[2 * si])
            c.ds(g + "/max", one * border[2 * si + 2])

    # ---- Rama map potential (synthetic maps; see module docstring)
    # maps get their own stream so a config is the same whether or not the
    # caller supplies coordinates
    def rama_maps(sq):
        return synthetic_rama_maps(list(sq), np.random.RandomState(seed + 104729))
    g = c.grp("rama_map_pot", ["rama_coord"], integrator_level=0)
    if tc is None:
        maps = rama_maps(seq_cpr)
        c.ds(g + "/residue_id", np.arange(n_res))
        c.ds(g + "/rama_map_id", np.arange(n_res))
        c.ds(g + "/rama_pot", maps)
    else:
        # trans-cis prolines leave the plain map for the trans and cis maps,
        # mixed by omega switches (write_rama_map_pot2)
        res_tc = tc[0]
        n_pro = len(res_tc)
        seq_trans, seq_cis = seq_cpr.copy(), seq_cpr.copy()
        seq_trans[res_tc], seq_cis[res_tc] = 'PRO', 'CPR'
        maps, maps_cis = rama_maps(seq_trans), rama_maps(seq_cis)
        rest = np.array([r for r in range(n_res) if r not in set(res_tc.tolist())], dtype=int)
        c.ds(g + "/residue_id", rest)
        c.ds(g + "/rama_map_id", rest)
        c.ds(g + "/rama_map_id_all", np.arange(n_res))
        c.ds(g + "/rama_pot", maps)
        ar = np.arange(n_pro)
        for nm, cen, sign in (("trans1", -0.5, 1.), ("trans2", 0.5, -1.), ("cis1", -0.5, -1.), ("cis2", 0.5, 1.)):
            g = c.grp("SigmoidCoord_" + nm, ["Dihedral_OmegaTransCis"], dim1=0)
            c.ds(g + "/id", ar)
            c.ds(g + "/c", np.ones(n_pro) * cen * np.pi)
            c.ds(g + "/s", np.ones(n_pro) * 3.0 / np.pi)
            c.ds(g + "/sign", np.ones(n_pro) * sign)
        for op, nm in (("Add", "trans"), ("Multiply", "cis")):
            g = c.grp("%s_lambda_%s" % (op, nm), ["SigmoidCoord_%s1" % nm, "SigmoidCoord_%s2" % nm],
                      n_dim=1, n_size=n_pro)
            for dsn in ("dim1", "dim2"):
                c.ds(g + "/" + dsn, np.array([0]))
            for dsn in ("id_pos1", "id_pos2", "id1_out", "id2_out"):
                c.ds(g + "/" + dsn, ar)
        for nm, op, mp in (("trans", "Add", maps), ("cis", "Multiply", maps_cis)):
            g = c.grp("RamaMap2_" + nm, ["rama_coord", "%s_lambda_%s" % (op, nm)], integrator_level=0)
            c.ds(g + "/residue_id", res_tc)
            c.ds(g + "/rama_map_id", res_tc)
            c.ds(g + "/rama_pot", mp)

    ref = np.log(P["rama_reference"])
    ref -= ref.mean()
    g = c.grp("rama_map_pot_ref", ["rama_coord"], log_pot=0)
    c.ds(g + "/residue_id", np.arange(n_res))
    c.ds(g + "/rama_map_id", np.zeros(n_res, dtype=np.int32))
    c.ds(g + "/rama_pot", ref[None])

    # ---- backbone steric pairs
    ref_pos = np.zeros((n_res, 4, 3))
    ref_pos[:, 0] = (-1.19280531, -0.83127186, 0.)
    ref_pos[:, 1] = (0., 0., 0.)
    ref_pos[:, 2] = (1.25222632, -0.87268266, 0.)
    ref_pos[:, 3] = (0., 0.94375626, 1.2068012)
    ref_pos[c.seq == 'GLY', 3] = np.nan
    ref_pos -= ref_pos[:, :3].mean(axis=1)[:, None]
    g = c.grp("backbone_pairs", ["affine_alignment"], integrator_level=1)
    c.ds(g + "/id", np.arange(n_res))
    c.ds(g + "/ref_pos", ref_pos)
    c.ds(g + "/n_atom", np.isfinite(ref_pos.sum(axis=-1)).sum(axis=-1))

    # ---- hydrogen bonds: infer_H_O, protein_hbond, hbond_energy
    excluded = set()
    for s in chain_first_residue:
        excluded.update([s - 1, s])
    donors = np.array([i for i in range(n_res) if i > 0 and i not in excluded and seq[i] != 'PRO'])
    acceptors = np.array([i for i in range(n_res) if i < n_res - 1 and i not in excluded])
    n_don, n_acc = len(donors), len(acceptors)
    g = c.grp("infer_H_O", ["pos"])
    c.ds(g + "/donors/residue", donors)
    c.ds(g + "/acceptors/residue", acceptors)
    c.ds(g + "/donors/bond_length", 0.88 * np.ones(n_don))
    c.ds(g + "/acceptors/bond_length", 1.24 * np.ones(n_acc))
    c.ds(g + "/donors/id", np.array((-1, 0, 1))[None, :] + 3 * donors[:, None])
    c.ds(g + "/acceptors/id", np.array((1, 2, 3))[None, :] + 3 * acceptors[:, None])

    g = c.grp("protein_hbond", ["infer_H_O"])
    c.ds(g + "/index1", np.arange(n_don))
    c.ds(g + "/type1", np.zeros(n_don, dtype=np.int32))
    c.ds(g + "/id1", donors)
    c.ds(g + "/index2", np.arange(n_don, n_don + n_acc))
    c.ds(g + "/type2", np.zeros(n_acc, dtype=np.int32))
    c.ds(g + "/id2", acceptors)
    c.ds(g + "/interaction_param", np.array([[[1.4, 1. / 0.10, 2.5, 1. / 0.125, 0.682, 1. / 0.05, 0., 0.]]]))

    g = c.grp("hbond_energy", ["protein_hbond", "rama_coord"], integrator_level=1)
    c.ds(g + "/parameters", P["hbond_parameter"])
    c.ds(g + "/donor_resid", donors)
    c.ds(g + "/acceptor_resid", acceptors)
    c.ds(g + "/rama_resid", np.arange(n_res))

    # ---- rotamer placement (fixed placement, dynamic 1-body)
    restype_num = {a.decode(): i for i, a in enumerate(P["sc_restype_order"])}
    placement_pos = P["sc_rotamer_center_fixed"]
    placement_energy = -np.log(P["sc_rotamer_prob"].transpose((2, 0, 1)))[..., None]
    start_stop = P["sc_rotamer_start_stop_bead"]
    rama_residue, affine_residue, layer_index, beadtype_seq, id_seq = [], [], [], [], []
    count_by_n_rot = {}
    for rnum, aa in enumerate(seq):
        start, stop, n_bead = start_stop[restype_num[aa]]
        n_rot = (stop - start) // n_bead
        if rnum in fix:
            # a fixed residue keeps the beads of its one state
            if not (0 <= fix[rnum] < n_rot):
                raise ValueError('invalid fix rotamer state')
            start, stop = start + n_bead * fix[rnum], start + n_bead * (fix[rnum] + 1)
            n_rot = 1
        count_by_n_rot.setdefault(n_rot, 0)
        base_id = (count_by_n_rot[n_rot] << N_BIT_ROTAMER) + n_rot
        count_by_n_rot[n_rot] += 1
        rama_residue.extend([rnum] * (stop - start))
        affine_residue.extend([rnum] * (stop - start))
        layer_index.extend(np.arange(start, stop))
        beadtype_seq.extend(['%s_%i' % (aa, i) for i in range(n_bead)] * n_rot)
        id_seq.extend(np.arange(stop - start) // n_bead + (base_id << N_BIT_ROTAMER))
    n_sc = len(affine_residue)
    sc_name, pl_name = "placement_fixed_point_vector_only", "placement_scalar"
    g = c.grp(sc_name, ["affine_alignment"])
    c.ds(g + "/rama_residue", np.array(rama_residue))
    c.ds(g + "/affine_residue", np.array(affine_residue))
    c.ds(g + "/layer_index", np.array(layer_index))
    c.ds(g + "/placement_data", placement_pos[..., :6])
    c.ds(g + "/beadtype_seq", np.array([b.encode() for b in beadtype_seq]))
    c.ds(g + "/id_seq", np.array(id_seq))
    if fix:
        c.ds(g + "/fix_rotamer", np.array(sorted(fix.items())))
    g = c.grp(pl_name, ["affine_alignment", "rama_coord"])
    c.ds(g + "/rama_residue", np.array(rama_residue))
    c.ds(g + "/affine_residue", np.array(affine_residue))
    c.ds(g + "/layer_index", np.array(layer_index))
    c.ds(g + "/placement_data", placement_energy.astype(np.float32))

    # ---- side chain / backbone coverage
    bead_num = {k.decode(): i for i, k in enumerate(P["sc_bead_order"])}
    sc_type = np.array([bead_num[s] for s in beadtype_seq])
    num_group = len(set(BACKBONE_GROUP4.values()))

    def bb_group(resid):
        bbt = BACKBONE_GROUP4[seq[resid]]
        if resid < n_res - 1 and seq[resid + 1] == 'PRO':
            bbt = num_group
        return bbt

    hb_type = [bb_group(r) * 2 + 0 for r in donors] + [bb_group(r) * 2 + 1 for r in acceptors]
    big = n_res > 1000
    g = c.grp("hbond_coverage", ["protein_hbond", sc_name], **({"max_n_edge": n_res * 80} if big else {}))
    c.ds(g + "/interaction_param", P["sc_coverage_interaction"])
    c.ds(g + "/index1", np.arange(n_don + n_acc))
    c.ds(g + "/type1", np.array(hb_type))
    c.ds(g + "/id1", np.concatenate([donors, acceptors]))
    c.ds(g + "/index2", np.arange(n_sc))
    c.ds(g + "/type2", sc_type)
    c.ds(g + "/id2", np.array(affine_residue))

    bb_index = np.arange(3 * n_res)
    g = c.grp("placement_fixed_point_vector_scalar", ["affine_alignment"])
    c.ds(g + "/affine_residue", bb_index // 3)
    c.ds(g + "/layer_index", bb_index % 3)
    c.ds(g + "/placement_data", P["sc_hydrophobe_placement"])
    g = c.grp("hbond_coverage_hydrophobe", ["placement_fixed_point_vector_scalar", sc_name],
              **({"max_n_edge": n_res * 120} if big else {}))
    c.ds(g + "/interaction_param", P["sc_hydrophobe_interaction"])
    c.ds(g + "/index1", bb_index)
    c.ds(g + "/type1", np.array([bb_group(r) * 3 + i for r in range(n_res) for i in range(3)]))
    c.ds(g + "/id1", bb_index // 3)
    c.ds(g + "/index2", np.arange(n_sc))
    c.ds(g + "/type2", sc_type)
    c.ds(g + "/id2", np.array(affine_residue))

    # ---- rotamer BP node
    g = c.grp("rotamer", [sc_name, pl_name, "hbond_coverage", "hbond_coverage_hydrophobe"],
              integrator_level=1, max_iter=1000, tol=bp_tol, damping=damping, iteration_chunk_size=2)
    pg = g + "/pair_interaction"
    w.group(pg)
    if big:
        w.set_attr(pg, "max_n_edge", n_res * 200)
    c.ds(pg + "/interaction_param", P["sc_pair_interaction"])
    c.ds(pg + "/index", np.arange(n_sc))
    c.ds(pg + "/type", sc_type)
    c.ds(pg + "/id", np.array(id_seq))

    # ---- environment
    env_order = {x.decode(): i for i, x in enumerate(P["env_restype_order"])}
    weights = P["env_weights"]
    cb = np.zeros((4, 3))
    cb[0] = (-1.19280531, -0.83127186, 0.)
    cb[2] = (1.25222632, -0.87268266, 0.)
    cb[3] = (0., 0.94375626, 1.2068012)
    cb -= cb[:3].mean(axis=0, keepdims=True)
    pdata = np.zeros((1, 6))
    pdata[0, 0:3] = cb[3]
    pdata[0, 3:6] = (cb[3] - cb[1]) / np.sqrt(((cb[3] - cb[1]) ** 2).sum())
    g = c.grp("placement_fixed_point_vector_only_CB", ["affine_alignment"])
    c.ds(g + "/affine_residue", np.arange(n_res))
    c.ds(g + "/layer_index", np.zeros(n_res, dtype=np.int32))
    c.ds(g + "/placement_data", pdata)

    aa_types = np.array([env_order[s] for s in seq])
    g = c.grp("environment_coverage_sc", ["placement_fixed_point_vector_only_CB", "weighted_pos"],
              num_aa_types=20, **({"max_n_edge": n_res * 160} if big else {}))
    c.ds(g + "/index1", np.arange(n_res))
    c.ds(g + "/type1", aa_types)
    c.ds(g + "/id1", np.arange(n_res))
    c.ds(g + "/index2", np.arange(n_sc))
    c.ds(g + "/type2", np.zeros(n_sc, dtype=np.int64))
    c.ds(g + "/id2", np.array(affine_residue))
    c.ds(g + "/interaction_param", P["env_coverage_param"])
    c.ds(g + "/aa_types", aa_types)

    method = "nonlinear" if environment_potential_type == 0 else "sigmoid"
    g = c.grp("%s_coupling_environment" % method, ["environment_coverage_sc"], integrator_level=1,
              number_independent_weights=20)
    c.ds(g + "/coupling_types", aa_types)
    c.ds(g + "/weights", weights)
    if environment_potential_type == 0:
        c.ds(g + "/coeff", P["env_energies"])
        w.set_attr(g + "/coeff", "spline_offset", P["env_energies_offset"])
        w.set_attr(g + "/coeff", "spline_inv_dx", P["env_energies_inv_dx"])
    else:
        c.ds(g + "/scale", P["env_scale"])
        c.ds(g + "/center", P["env_center"])
        c.ds(g + "/sharpness", P["env_sharpness"])

    res_id = np.concatenate([donors, acceptors])
    g = c.grp("environment_coverage_hb", ["infer_H_O", "weighted_pos"], num_aa_types=20,
              **({"max_n_edge": n_res * 160} if big else {}))
    c.ds(g + "/interaction_param", np.array([[[6.0, 1.0, -0.1, 1.0]]]))
    c.ds(g + "/aa_types", np.array([env_order[seq[i]] for i in res_id]))
    c.ds(g + "/index1", np.arange(n_don + n_acc))
    c.ds(g + "/type1", np.zeros(n_don + n_acc, dtype=np.int64))
    c.ds(g + "/id1", res_id)
    c.ds(g + "/index2", np.arange(n_sc))
    c.ds(g + "/type2", np.zeros(n_sc, dtype=np.int64))
    c.ds(g + "/id2", np.array(affine_residue))

    for name, i1, t1, i2, t2 in (("hb_environment_coverage_hn", np.arange(n_don), donors,
                                  np.arange(n_don, n_don + n_acc), acceptors),
                                 ("hb_environment_coverage_oc", np.arange(n_don, n_don + n_acc), acceptors,
                                  np.arange(n_don), donors)):
        g = c.grp(name, ["infer_H_O", "infer_H_O"], **({"max_n_edge": n_res * 6} if big else {}))
        c.ds(g + "/interaction_param", np.array([[[3.5, 2.0, 0.0, 2.0]]]))
        c.ds(g + "/index1", i1)
        c.ds(g + "/type1", np.zeros(len(i1), dtype=np.int64))
        c.ds(g + "/id1", t1)
        c.ds(g + "/index2", i2)
        c.ds(g + "/type2", np.zeros(len(i2), dtype=np.int64))
        c.ds(g + "/id2", t2)

    g = c.grp("cat_pos_bb_coverage", ["hb_environment_coverage_hn", "hb_environment_coverage_oc"], n_dim=1)
    c.ds(g + "/index_pos1", np.arange(n_don))
    c.ds(g + "/index_pos2", np.arange(n_acc))

    bb_env = P["bb_env"]
    g = c.grp("bb_sigmoid_coupling_environment", ["environment_coverage_hb", "cat_pos_bb_coverage"],
              integrator_level=1, num_aa_types=20, scale=bb_env[0], center=bb_env[1],
              sharpness=bb_env[2], hbond_weight=bb_env[3])
    c.ds(g + "/weights", weights)

    g = c.grp("weighted_pos", [sc_name, pl_name])
    c.ds(g + "/index_pos", np.arange(n_sc))
    c.ds(g + "/index_weight", np.arange(n_sc))

    # ---- rama coordinates and rigid frames
    N_id = 3 * np.arange(n_res)
    id1 = np.column_stack((N_id - 1, N_id, N_id + 1, N_id + 2))
    id2 = np.column_stack((N_id, N_id + 1, N_id + 2, N_id + 3))
    id2[id2 >= n_atom] = -1
    id3 = np.column_stack((N_id - 1, N_id, N_id + 1, N_id + 2, N_id + 3))
    id3[id3 >= n_atom] = -1
    if c.n_chains > 1:
        for loc in range(n_res):
            ids = id3[loc]
            chain = (ids[:, None] >= c.chain_starts).sum(axis=-1)
            if not (ids >= 0).all() or (chain == chain[0]).all():
                if ids[0] >= 0 and ids[4] >= 0:
                    continue
            if chain[0] != chain[1] and ids[0] >= 0:
                id3[loc, 0] = -1
                id1[loc, 0] = -1
            if ids[4] >= 0 and chain[3] != chain[4]:
                id3[loc, 4] = -1
                id2[loc, 3] = -1
    g = c.grp("Dihedral_phi", ["pos"])
    c.ds(g + "/id", id1)
    g = c.grp("Dihedral_psi", ["pos"])
    c.ds(g + "/id", id2)
    g = c.grp("rama_coord", ["Dihedral_phi", "Dihedral_psi"])
    c.ds(g + "/index_pos1", np.arange(n_res))
    c.ds(g + "/index_pos2", np.arange(n_res))
    c.ds(g + "/id", id3)

    ref_geom = np.zeros((n_res, 3, 3))
    ref_geom[:, 0] = (-1.19280531, -0.83127186, 0.)
    ref_geom[:, 2] = (1.25222632, -0.87268266, 0.)
    ref_geom -= ref_geom.mean(axis=1)[:, None]
    g = c.grp("affine_alignment", ["pos"])
    c.ds(g + "/atoms", np.column_stack((N_id, N_id + 1, N_id + 2)))
    c.ds(g + "/ref_geom", ref_geom)

    if (surface is not None or channel_membrane or lateral_pressure is not None) and membrane_thickness is None:
        raise ValueError("the surface and channel/lateral membrane terms need membrane_thickness")
    if (channel_membrane or lateral_pressure is not None) and surface is None:
        raise ValueError("the channel and lateral membrane terms need the surface node")
    if membrane_thickness is not None:
        half = 0.5 * membrane_thickness
        names = [x.decode() for x in P["mem_names"]]
        cb_e, hb_e, nodes = P["mem_cb_energy"], P["mem_hb_energy"], P["mem_burial_nodes"]
        if nodes.size + 1 != cb_e.shape[1]:
            raise ValueError("burial nodes do not match the membrane energy table")
        cb_dz = (P["mem_cb_z_max"] - P["mem_cb_z_min"]) / (cb_e.shape[2] - 2)
        hb_dz = (P["mem_hb_z_max"] - P["mem_hb_z_min"]) / (hb_e.shape[2] - 2)
        g = c.grp("Const3D_curvature_center", ["pos"], dim1=0, dim2=1, dim3=2, initialized_by_coord=0)
        c.ds(g + "/id", np.arange(1))
        c.ds(g + "/value", np.array([[0., 0., curvature_radius * -1 * curvature_sign]]))
        common = dict(integrator_level=0, left_right_node=0.0, half_thickness=half, use_curvature=int(use_curvature),
                      curvature_radius=curvature_radius, curvature_sign=curvature_sign)
        surf = "surf_" if channel_membrane else ""
        cb_args = ["placement_fixed_point_only_CB", "environment_coverage_sc"] + (["surface"] if surf else [])
        g = c.grp("cb_%smembrane_potential" % surf, cb_args + ["Const3D_curvature_center"],
                  z_start=P["mem_cb_z_min"] - half, z_scale=1. / cb_dz, bl_range_sharpness=1.0,
                  left_right_sharpness=1. / cb_dz, **common)
        used = np.array([r for r in range(n_res) if r not in set(membrane_exclude_residues)], dtype=int)
        res_type = np.array([names.index(seq[r]) for r in used], dtype=int)
        c.ds(g + "/cb_index", used)
        c.ds(g + "/res_type", res_type)
        c.ds(g + "/weights", weights[:20])
        c.ds(g + "/bl_nodes", nodes)
        c.ds(g + "/coeff", cb_e)
        if surf:
            c.ds(g + "/coeff_inner", P["mem_icb_energy"])
        hb_args = ["protein_hbond"] + (["environment_coverage_sc", "surface"] if surf else [])
        g = c.grp("hb_%smembrane_potential" % surf, hb_args + ["Const3D_curvature_center"],
                  z_start=P["mem_hb_z_min"] - half, z_scale=1. / hb_dz, left_right_sharpness=1. / hb_dz, **common)
        res_hb = np.concatenate([donors, acceptors])
        hb_used = np.array([i for i, r in enumerate(res_hb) if r not in excluded], dtype=int)
        hb_type = np.concatenate([np.zeros(n_don, dtype='i'), np.ones(n_acc, dtype='i')])
        c.ds(g + "/hb_index", hb_used)
        c.ds(g + "/coeff", hb_e)
        if surf:
            # one type and residue per used entry (the reference's checks want
            # hb_type and hb_res as long as hb_index)
            c.ds(g + "/hb_type", hb_type[hb_used])
            c.ds(g + "/hb_res", res_hb[hb_used].astype(int))
            c.ds(g + "/weights", weights[:20])
            c.ds(g + "/coeff_inner", P["mem_ihb_energy"])
        else:
            c.ds(g + "/hb_type", hb_type)
        ref_cb = np.zeros((4, 3))
        ref_cb[0] = (-1.19280531, -0.83127186, 0.)
        ref_cb[2] = (1.25222632, -0.87268266, 0.)
        ref_cb[3] = (0., 0.94375626, 1.2068012)
        ref_cb -= ref_cb[:3].mean(axis=0, keepdims=True)
        g = c.grp("placement_fixed_point_only_CB", ["affine_alignment"])
        c.ds(g + "/affine_residue", np.arange(n_res))
        c.ds(g + "/layer_index", np.zeros(n_res, dtype='i'))
        c.ds(g + "/placement_data", ref_cb[3][None])
        if surface is not None:
            _write_surface(c, n_res, int(surface), half, surface_included_residues)
        if lateral_pressure is not None:
            attrs, pp = _lateral_spline(lateral_pressure, half)
            g = c.grp("membranelateral_potential", ["placement_fixed_point_only_CB", "environment_coverage_sc", "surface"],
                      **attrs)
            c.ds(g + "/cb_index", used)
            c.ds(g + "/restypes", res_type)
            c.ds(g + "/weights", weights[:20])
            c.ds(g + "/cov_midpoint", np.ones(20) + 2.5)
            c.ds(g + "/cov_sharpness", np.ones(20))
            c.ds(g + "/params", pp)

    for name, args, attrs, dsets in extra_nodes:
        g = c.grp(name, args, **attrs)
        for k, v in dsets.items():
            c.ds(g + "/" + k, np.asarray(v))

    if moves:
        if c.n_chains > 1:
            starts = np.append(c.chain_starts, n_atom)
            ranges = np.array([[starts[i], starts[i + 1]] for i in range(c.n_chains)], dtype=np.int32)
            w.dataset("/input/jump_moves/atom_range", ranges)
            w.dataset("/input/jump_moves/sigma_trans", np.full(len(ranges), jump_length_scale, dtype=np.float32))
            w.dataset("/input/jump_moves/sigma_rot",
                      np.full(len(ranges), jump_rotation_scale * np.pi / 180., dtype=np.float32))
        else:
            inner = np.array([-1 not in tuple(x) for x in id3])
            piv = id3[inner]
            w.dataset("/input/pivot_moves/proposal_pot", maps)
            w.dataset("/input/pivot_moves/pivot_atom", piv.astype(np.int32))
            w.dataset("/input/pivot_moves/pivot_restype", np.arange(maps.shape[0])[inner].astype(np.int32))
            w.dataset("/input/pivot_moves/pivot_range",
                      np.column_stack((piv[:, 4] + 1, np.full(len(piv), n_atom))).astype(np.int32))

    w.save(path)
    return np.asarray(pos, dtype=np.float32)


# points on the circle of an atom's radius, in units of the radius, that
# fill the voxels around each atom (write_surface_coord's table,
# py/upside_config.py:1557-1575: the 6 directions of a hexagon at radius 1 and
# 1/2 and the 6 midpoints between them at radius sqrt(3)/2)
def _surface_aux_points():
    pts = []
    for k in range(6):
        a = np.pi / 2 - k * np.pi / 3
        pts.append((round(np.cos(a), 3), round(np.sin(a), 3)))
        pts.append((round(0.5 * np.cos(a), 3), round(0.5 * np.sin(a), 3)))
    for k in range(6):
        a = np.pi / 3 - k * np.pi / 3
        pts.append((round(0.866 * np.cos(a), 3), round(0.866 * np.sin(a), 3)))
    return np.array(pts, dtype=np.float64) + 0.0


def _write_surface(c, n_res, method, half, included):
    if method not in (0, 1):
        raise ValueError("surface method must be 0 (fast) or 1 (lipid diffusion)")
    g = c.grp("cat_pos_bb_cb", ["pos", "placement_fixed_point_only_CB"], n_dim=3)
    c.ds(g + "/index_pos1", np.arange(3 * n_res))
    c.ds(g + "/index_pos2", np.arange(n_res))
    attrs = dict(n_rotation=20, half_thickness=half, zbuffer=0.0, exclusion=1 if len(included) else 0,
                 len_gridx=3.0, len_gridy=3.0, n_gridz=6, n_smallgridx=1, n_smallgridy=1, n_smallgridz=2,
                 atom_radius=1.6, method_type=method)
    g = c.grp("surface", ["cat_pos_bb_cb"], **attrs)
    if len(included):
        c.ds(g + "/included_list", np.array(included, dtype=int))
    c.ds(g + "/index_cb", np.arange(n_res) + 3 * n_res)
    c.ds(g + "/auxiliary_point", _surface_aux_points())


def clamped_spline_solve(values):
    """B-spline coefficients (len(values) + 2, float32) of the clamped spline
    through `values` at the integer knots with zero end slopes: the
    reference's clamped_spline_solve (src/spline.cpp:158-190, called through
    py/upside_engine.py:138-150), a tridiagonal solve in double precision."""
    d = np.asarray(values, dtype=np.float32).astype(np.float64)
    n = d.size
    if n < 2:
        raise ValueError("clamped spline needs at least 2 values")
    a = np.full(n, 1. / 6.)
    b = np.full(n, 2. / 3.)
    cc = np.full(n, 1. / 6.)
    cc[0] *= 2.
    a[n - 1] *= 2.
    for k in range(1, n):
        m = a[k] / b[k - 1]
        b[k] -= m * cc[k - 1]
        d[k] -= m * d[k - 1]
    d[n - 1] /= b[n - 1]
    for k in range(n - 2, -1, -1):
        d[k] = (d[k] - cc[k] * d[k + 1]) / b[k]
    out = np.zeros(n + 2, dtype=np.float32)
    out[1:n + 1] = d
    out[0] = out[2]
    out[n + 1] = out[n - 1]
    return out


def read_lateral_pressure(table):
    """(z, pressure) rows of a --membrane-lateral-potential table: a path to
    a text file whose first line is "z lateral_pressure", or the rows."""
    if not isinstance(table, str):
        return np.asarray(table, dtype=float).reshape(-1, 2)
    with open(table) as fh:
        rows = [ln.split() for ln in fh if ln.strip()]
    if [x.lower() for x in rows[0]] != ["z", "lateral_pressure"]:
        raise ValueError('First line must be "z lateral_pressure"')
    if not all(len(r) == 2 for r in rows):
        raise ValueError("Invalid format")
    return np.asarray(rows[1:], dtype=float).reshape(-1, 2)


def _lateral_spline(table, half):
    """Attributes and spline coefficients of membranelateral_potential.  The
    pressure curve is interpolated by a cubic spline held constant beyond its
    ends, sampled at 1 angstrom knots over [min z, max z] and fitted by the
    clamped spline."""
    import scipy.interpolate
    f = read_lateral_pressure(table)
    z0, p0 = f[:, 0], f[:, 1]
    spl = scipy.interpolate.InterpolatedUnivariateSpline(z0, p0)
    min_z, max_z = float(np.min(z0)), float(np.max(z0))
    n_knot = int(max_z - min_z) + 1
    z = np.linspace(min_z, max_z, n_knot)
    vals = np.select([z < z0[0], z > z0[-1], np.ones_like(z, dtype=bool)],
                     [np.zeros_like(z) + p0[0], np.zeros_like(z) + p0[-1], spl(z)])
    pp = clamped_spline_solve(vals)
    return dict(min_z=min_z, max_z=max_z, inv_dz=1. / (max_z - min_z), n_knot=len(pp), half_thickness=half,
                integrator_level=0), pp


def random_sequence(n_res, rng):
    return [AA[i] for i in rng.randint(0, 20, size=n_res)]
