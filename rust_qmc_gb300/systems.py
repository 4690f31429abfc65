"""System descriptions for the walker path.

A ``SystemSpec`` holds, as numpy arrays, exactly what ``qmc_system_desc``
carries: nuclei, a basis of contracted Gaussian or Slater-type AOs, MO
coefficients, the electrons' spins and Slater columns, and the Jastrow.

Builders:
  * ``h2_mo``            H2 LCAO, src/systems/hydrogen.rs:28-35,115-200
  * ``lithium_atom``     Li STO-7G x Jastrow2, src/systems/lithium.rs, src/main.rs:34-49
  * ``methane_gto``      CH4 6-31G x Jastrow3, src/systems/methane.rs:600-776
  * ``methane_minimal``  the 9-function CH4 with seeded QR-orthonormal MOs
                         (65 536-walker single-electron workload)
  * ``benzene_minimal``  planar C6H6, 42 electrons, 36 contracted Gaussians,
                         seeded QR-orthonormal MOs (16 384-walker VMC/DMC workload)
  * ``benzene_gto``      BenzeneGTO: 6-31G (66 AOs), the hand-built MO table,
                         src/systems/benzene.rs:48-470
  * ``electron_gas``     periodic homogeneous electron gas, src/systems/heg.rs
"""
import ctypes as C
import math

import numpy as np

from . import _lib as L

# ---------------------------------------------------------------------------
# Basis data restated from the reference's tables.
# ---------------------------------------------------------------------------
# STO-7G Li radial functions, src/wavefunction/slater.rs:68-89.
LI_STO_EXPONENTS = [0.72089388, 2.61691643, 0.69257443, 1.37137558, 3.97864549, 13.52900016, 19.30801440]
LI_STO_POWERS = [1, 1, 2, 2, 2, 2, 3]
LI_STO_1S = [-0.12220686, 1.11273225, 0.04125378, 0.09306499, -0.10260021, -0.00034191, 0.00021963]
LI_STO_2S = [0.47750469, 0.11140449, -1.25954273, -0.18475003, -0.02736293, -0.00025064, 0.00057962]

# 6-31G primitives, src/systems/methane.rs:701-770 (raw coefficients).
C_1S = [(3047.5249, 0.0018347), (457.36951, 0.0140373), (103.94869, 0.0688426),
        (29.210155, 0.2321844), (9.2866630, 0.4679413), (3.1639270, 0.3623120)]
C_SP_INNER_EXP = [7.8682724, 1.8812885, 0.5442493]
C_SP_INNER_S = [-0.1193324, -0.1608542, 1.1434564]
C_SP_INNER_P = [0.0689991, 0.3164240, 0.7443083]
C_SP_OUTER_EXP = 0.1687145
H_INNER = [(18.7311370, 0.0334946), (2.8253937, 0.2347270), (0.6401217, 0.8137573)]
H_OUTER_EXP = 0.1612778

# RHF/6-31G MO table of MethaneGTO, src/systems/methane.rs:662-674.
METHANE_GTO_MO = [
    [0.9943, 0.0234, 0.0, 0.0, 0.0, 0.0020, 0.0, 0.0, 0.0, 0.0018, 0.0018, 0.0018, 0.0018, 0.0015, 0.0015, 0.0015, 0.0015],
    [-0.0237, 0.2223, 0.0, 0.0, 0.0, 0.8340, 0.0, 0.0, 0.0, 0.0673, 0.0673, 0.0673, 0.0673, 0.0437, 0.0437, 0.0437, 0.0437],
    [0.0, 0.0, 0.2090, 0.0, 0.0, 0.0, 0.5730, 0.0, 0.0, 0.1020, 0.1020, -0.1020, -0.1020, 0.0670, 0.0670, -0.0670, -0.0670],
    [0.0, 0.0, 0.0, 0.2090, 0.0, 0.0, 0.0, 0.5730, 0.0, 0.1020, -0.1020, 0.1020, -0.1020, 0.0670, -0.0670, 0.0670, -0.0670],
    [0.0, 0.0, 0.0, 0.0, 0.2090, 0.0, 0.0, 0.0, 0.5730, 0.1020, -0.1020, -0.1020, 0.1020, 0.0670, -0.0670, -0.0670, 0.0670],
]

CH_BOND = 2.05           # bohr, src/systems/methane.rs:23
SEED_BASE = 0x51A7E5     # seeds of the synthetic workloads: SEED_BASE + workload number


def tetrahedral_ch4(bond=CH_BOND):
    """C at the origin, H at (+-d,+-d,+-d) with even parity (methane.rs:625-632)."""
    d = bond / math.sqrt(3.0)
    return np.array([[0, 0, 0], [d, d, d], [d, -d, -d], [-d, d, -d], [-d, -d, d]], dtype=np.float64)


# ---------------------------------------------------------------------------
# Seeded normals from Philox4x32-10 (the same generator the kernels use), so
# synthetic MO tables are reproducible on any platform.
# ---------------------------------------------------------------------------
_M0, _M1, _W0, _W1 = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85
_MASK = 0xFFFFFFFF


def philox4x32(ctr, key):
    """Philox4x32-10 (Salmon et al., SC'11) on Python integers."""
    c0, c1, c2, c3 = ctr
    k0, k1 = key
    for r in range(10):
        if r:
            k0 = (k0 + _W0) & _MASK
            k1 = (k1 + _W1) & _MASK
        p0 = _M0 * c0
        p1 = _M1 * c2
        c0, c1, c2, c3 = ((p1 >> 32) ^ c1 ^ k0) & _MASK, p1 & _MASK, ((p0 >> 32) ^ c3 ^ k1) & _MASK, p0 & _MASK
    return c0, c1, c2, c3


def seeded_normals(seed, n, stream=0xA0):
    """n standard normals from Philox keyed by ``seed`` (Box-Muller pairs)."""
    out = []
    i = 0
    key = (seed & _MASK, (seed >> 32) & _MASK)
    while len(out) < n:
        x = philox4x32((i, 0, 0, stream), key)
        for a, b in ((x[0], x[1]), (x[2], x[3])):
            u1 = (a + 0.5) / 4294967296.0
            u2 = (b + 0.5) / 4294967296.0
            r = math.sqrt(-2.0 * math.log(u1))
            out.append(r * math.cos(2.0 * math.pi * u2))
            out.append(r * math.sin(2.0 * math.pi * u2))
        i += 1
    return np.array(out[:n], dtype=np.float64)


def seeded_orthonormal(seed, n):
    """Q of the QR factorisation (positive diagonal R) of a seeded n x n normal
    matrix, by modified Gram-Schmidt in FP64.  Columns are orthonormal."""
    A = seeded_normals(seed, n * n).reshape(n, n)
    Q = np.zeros((n, n))
    for j in range(n):
        v = A[:, j].copy()
        for i in range(j):
            v -= (Q[:, i] @ v) * Q[:, i]
        Q[:, j] = v / math.sqrt(v @ v)
    return Q


class SystemSpec:
    """Numpy-held system description; ``desc()`` returns the C struct."""

    def __init__(self, *, spins, nuc_pos, nuc_charge, basis_kind, ao_nuc, ao_l, ao_m, ao_prims,
                 mo_coef, occ, jastrow_kind, jas_F=1.0, jas=None, nuc_species=None,
                 rot_occ=(), rot_virt=(), rot_angle=(), quirks=0, init_nuc=None, init_sigma=0.5,
                 box_L=0.0, name="system"):
        self.name = name
        self.spins = np.ascontiguousarray(spins, dtype=np.int32)
        self.nuc_pos = np.ascontiguousarray(nuc_pos, dtype=np.float64).reshape(-1, 3)
        self.box_L = float(box_L)
        self.nuc_charge = np.ascontiguousarray(nuc_charge, dtype=np.float64)
        n_nuc = len(self.nuc_charge)
        self.nuc_species = np.ascontiguousarray(nuc_species if nuc_species is not None else [0] * n_nuc,
                                                dtype=np.int32)
        self.basis_kind = int(basis_kind)
        self.ao_nuc = np.ascontiguousarray(ao_nuc, dtype=np.int32)
        self.ao_l = np.ascontiguousarray(ao_l, dtype=np.int32)
        self.ao_m = np.ascontiguousarray(ao_m, dtype=np.int32)
        off, ex, cf, pw = [0], [], [], []
        for prims in ao_prims:        # list of (exp, coef[, pow])
            for p in prims:
                ex.append(p[0]); cf.append(p[1]); pw.append(p[2] if len(p) > 2 else 0)
            off.append(len(ex))
        self.ao_prim_off = np.array(off, dtype=np.int32)
        self.prim_exp = np.array(ex, dtype=np.float64)
        self.prim_coef = np.array(cf, dtype=np.float64)
        self.prim_pow = np.array(pw, dtype=np.int32)
        self.mo_coef = np.ascontiguousarray(mo_coef, dtype=np.float64)
        self.occ = np.ascontiguousarray(occ, dtype=np.int32)
        self.jastrow_kind = int(jastrow_kind)
        self.jas_F = float(jas_F)
        self.jas = np.zeros(8) if jas is None else np.array(jas, dtype=np.float64)
        self.rot_occ = np.ascontiguousarray(rot_occ, dtype=np.int32)
        self.rot_virt = np.ascontiguousarray(rot_virt, dtype=np.int32)
        self.rot_angle = np.ascontiguousarray(rot_angle, dtype=np.float64)
        self.quirks = int(quirks)
        self.init_nuc = np.ascontiguousarray(init_nuc if init_nuc is not None else [-1] * len(self.spins),
                                             dtype=np.int32)
        self.init_sigma = float(init_sigma)

    @property
    def n_elec(self):
        return len(self.spins)

    @property
    def n_nuc(self):
        return len(self.nuc_charge)

    @property
    def n_params(self):
        return 8 + len(self.rot_occ)

    def params(self):
        return np.concatenate([self.jas, self.rot_angle])

    def with_params(self, p):
        """Copy with the optimisable parameters replaced (jas[0..7], angles)."""
        s = self.copy()
        p = np.asarray(p, dtype=np.float64)
        s.jas = p[:8].copy()
        s.rot_angle = p[8:].copy()
        return s

    def with_nuclei(self, R):
        s = self.copy()
        s.nuc_pos = np.ascontiguousarray(R, dtype=np.float64).reshape(-1, 3)
        return s

    def copy(self):
        import copy
        return copy.deepcopy(self)

    def v_nn(self):
        if self.box_L > 0:
            return 0.0
        v = 0.0
        for I in range(self.n_nuc):
            for J in range(I + 1, self.n_nuc):
                v += self.nuc_charge[I] * self.nuc_charge[J] / np.linalg.norm(self.nuc_pos[I] - self.nuc_pos[J])
        return v

    def desc(self):
        """ctypes ``qmc_system_desc`` pointing into this object's arrays."""
        def ip(a):
            return a.ctypes.data_as(C.POINTER(C.c_int)) if a is not None and a.size else None

        def dp(a):
            return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None and a.size else None

        d = L.SystemDesc()
        d.n_elec = self.n_elec
        d.spins = ip(self.spins)
        d.n_nuc = self.n_nuc
        self._pos_flat = np.ascontiguousarray(self.nuc_pos.reshape(-1))
        d.nuc_pos = dp(self._pos_flat)
        d.nuc_charge = dp(self.nuc_charge)
        d.nuc_species = ip(self.nuc_species)
        d.basis_kind = self.basis_kind
        d.n_ao = len(self.ao_nuc)
        d.ao_nuc, d.ao_l, d.ao_m, d.ao_prim_off = ip(self.ao_nuc), ip(self.ao_l), ip(self.ao_m), ip(self.ao_prim_off)
        d.prim_exp, d.prim_coef = dp(self.prim_exp), dp(self.prim_coef)
        d.prim_pow = ip(self.prim_pow) if self.basis_kind == L.QMC_BASIS_STO else None
        if not self.prim_exp.size:
            d.ao_prim_off = None
        d.n_mo = self.mo_coef.shape[0]
        self._mo_flat = np.ascontiguousarray(self.mo_coef.reshape(-1))
        d.mo_coef = dp(self._mo_flat)
        d.occ = ip(self.occ)
        d.jastrow_kind = self.jastrow_kind
        d.jas_F = self.jas_F
        for i in range(8):
            d.jas[i] = float(self.jas[i])
        d.n_rot = len(self.rot_occ)
        d.rot_occ, d.rot_virt, d.rot_angle = ip(self.rot_occ), ip(self.rot_virt), dp(self.rot_angle)
        d.quirks = self.quirks
        d.init_nuc = ip(self.init_nuc)
        d.init_sigma = self.init_sigma
        d.box_L = self.box_L
        return d


# ---------------------------------------------------------------------------
# Builders
# ---------------------------------------------------------------------------
def h2_mo(alpha=1.2, F=3.0, half_bond=0.7, init="nuclei", init_sigma=1.0):
    """H2 LCAO: psi = phi(r1) phi(r2) J(r12), phi = e^{-a|r-A|} + e^{-a|r-B|}.

    Nucleus 0 at (0,0,+half_bond), nucleus 1 at (0,0,-half_bond) as in
    conf/h2.yaml.  ``init="nuclei"`` places electron i at N(R_i, sigma) (the
    4096-walker workload); ``init="origin"`` is Jastrow1::initialize
    (src/correlation/jastrow.rs:21-28)."""
    R = [[0, 0, half_bond], [0, 0, -half_bond]]
    return SystemSpec(
        name="H2", spins=[1, -1], nuc_pos=R, nuc_charge=[1.0, 1.0], basis_kind=L.QMC_BASIS_STO,
        ao_nuc=[0, 1], ao_l=[0, 0], ao_m=[0, 0], ao_prims=[[(alpha, 1.0, 0)], [(alpha, 1.0, 0)]],
        mo_coef=[[1.0, 1.0]], occ=[0, 0], jastrow_kind=L.QMC_JAS_PADE_F, jas_F=F,
        init_nuc=[0, 1] if init == "nuclei" else [-1, -1], init_sigma=init_sigma)


def lithium_atom(F=1.0, reference_quirks=True):
    """Li: STOSlaterDet([1s, 1s, 2s], spins [+1,-1,+1]) x Jastrow2(F)
    (src/main.rs:37-48).  With ``reference_quirks`` the Jastrow2 gradient and
    Laplacian follow src/correlation/jastrow.rs:95-125 exactly."""
    prims = [(z, c, p) for z, c, p in zip(LI_STO_EXPONENTS, LI_STO_1S, LI_STO_POWERS)]
    prims2 = [(z, c, p) for z, c, p in zip(LI_STO_EXPONENTS, LI_STO_2S, LI_STO_POWERS)]
    return SystemSpec(
        name="Li", spins=[1, -1, 1], nuc_pos=[[0, 0, 0]], nuc_charge=[3.0], basis_kind=L.QMC_BASIS_STO,
        ao_nuc=[0, 0], ao_l=[0, 0], ao_m=[0, 0], ao_prims=[prims, prims2],
        mo_coef=np.eye(2), occ=[0, 0, 1], jastrow_kind=L.QMC_JAS_PADE_F, jas_F=F,
        quirks=(L.QMC_QUIRK_J2_GRAD | L.QMC_QUIRK_J2_LAP) if reference_quirks else 0,
        init_nuc=[-1, -1, -1], init_sigma=1.0)


def _gto_631g_ch4(R):
    """17 AOs of MethaneGTO::build_631g_basis (src/systems/methane.rs:697-776)."""
    ao_nuc, ao_l, ao_m, prims = [], [], [], []

    def add(n, l, m, p):
        ao_nuc.append(n); ao_l.append(l); ao_m.append(m); prims.append(p)

    add(0, 0, 0, C_1S)
    add(0, 0, 0, list(zip(C_SP_INNER_EXP, C_SP_INNER_S)))
    for m in range(3):
        add(0, 1, m, list(zip(C_SP_INNER_EXP, C_SP_INNER_P)))
    add(0, 0, 0, [(C_SP_OUTER_EXP, 1.0)])
    for m in range(3):
        add(0, 1, m, [(C_SP_OUTER_EXP, 1.0)])
    for h in range(4):
        add(1 + h, 0, 0, H_INNER)
    for h in range(4):
        add(1 + h, 0, 0, [(H_OUTER_EXP, 1.0)])
    return ao_nuc, ao_l, ao_m, prims


def jastrow3_params(b_ee, b_en, a_anti=0.5, a_para=0.25):
    """Reference Jastrow3 (src/correlation/jastrow.rs:165-185) in the
    generalised parameter vector {b_anti,b_para,a_anti,a_para,B0,B1,A0,A1}."""
    return [b_ee, b_ee, a_anti, a_para, b_en, b_en, 1.0, 1.0]


def reference_params_from_general(p):
    """Map the general vector back to MethaneGTO's 4 (b_ee,b_en,a_anti,a_para)."""
    return [p[0], p[4], p[2], p[3]]


def methane_gto(b_ee=1.5, b_en=2.0, bond=CH_BOND):
    """MethaneGTO (src/systems/methane.rs:623-685): 6-31G basis, fixed MO
    table, Jastrow3.  Electrons 0-4 spin up, 5-9 spin down."""
    R = tetrahedral_ch4(bond)
    ao_nuc, ao_l, ao_m, prims = _gto_631g_ch4(R)
    return SystemSpec(
        name="CH4-6-31G", spins=[1] * 5 + [-1] * 5, nuc_pos=R, nuc_charge=[6, 1, 1, 1, 1],
        nuc_species=[0, 1, 1, 1, 1], basis_kind=L.QMC_BASIS_GTO, ao_nuc=ao_nuc, ao_l=ao_l, ao_m=ao_m,
        ao_prims=prims, mo_coef=METHANE_GTO_MO, occ=[0, 1, 2, 3, 4] * 2, jastrow_kind=L.QMC_JAS_PADE_EEN,
        jas=jastrow3_params(b_ee, b_en),
        init_nuc=[0] * 6 + [1, 2, 3, 4], init_sigma=0.5)


def methane_minimal(seed=SEED_BASE + 2, b_ee=1.5, b_en=2.0, n_rot=4, bond=CH_BOND):
    """The 9-function CH4 workload: C 1s (the three most diffuse 6-31G C 1s
    primitives), C 2s and 2p (6-31G SP inner shell), four H 1s (6-31G H inner
    shell), every AO three primitives with the reference's raw coefficients.
    MO coefficients: columns of Q from QR of a seeded 9x9 normal matrix; MOs
    0-4 occupied in both spin sectors, MOs 5-8 are the virtuals that the
    ``n_rot`` mixing angles rotate into MOs 1..n_rot.  Jastrow3 form with a
    one-body (e-n) term, species C = 0, H = 1."""
    R = tetrahedral_ch4(bond)
    ao_nuc, ao_l, ao_m, prims = [], [], [], []
    ao_nuc.append(0); ao_l.append(0); ao_m.append(0); prims.append(C_1S[3:])
    ao_nuc.append(0); ao_l.append(0); ao_m.append(0); prims.append(list(zip(C_SP_INNER_EXP, C_SP_INNER_S)))
    for m in range(3):
        ao_nuc.append(0); ao_l.append(1); ao_m.append(m); prims.append(list(zip(C_SP_INNER_EXP, C_SP_INNER_P)))
    for h in range(4):
        ao_nuc.append(1 + h); ao_l.append(0); ao_m.append(0); prims.append(H_INNER)
    Q = seeded_orthonormal(seed, 9)
    mo = Q.T.copy()                      # row k = MO k = column k of Q
    rot_occ = list(range(1, 1 + n_rot))
    rot_virt = list(range(5, 5 + n_rot))
    return SystemSpec(
        name="CH4-min", spins=[1] * 5 + [-1] * 5, nuc_pos=R, nuc_charge=[6, 1, 1, 1, 1],
        nuc_species=[0, 1, 1, 1, 1], basis_kind=L.QMC_BASIS_GTO, ao_nuc=ao_nuc, ao_l=ao_l, ao_m=ao_m,
        ao_prims=prims, mo_coef=mo, occ=[0, 1, 2, 3, 4] * 2, jastrow_kind=L.QMC_JAS_PADE_EEN,
        jas=jastrow3_params(b_ee, b_en), rot_occ=rot_occ, rot_virt=rot_virt, rot_angle=[0.0] * n_rot,
        init_nuc=[0] * 6 + [1, 2, 3, 4], init_sigma=0.5)


def hexagonal_c6h6(cc=2.64, ch=2.05):
    """D6h benzene in the z = 0 plane (src/systems/benzene.rs:119-140):
    carbons on a hexagon of radius C-C, hydrogens radially outward at C-C + C-H."""
    C, H = [], []
    for i in range(6):
        a = math.pi / 3.0 * i
        C.append([cc * math.cos(a), cc * math.sin(a), 0.0])
        H.append([(cc + ch) * math.cos(a), (cc + ch) * math.sin(a), 0.0])
    return np.array(C + H, dtype=np.float64)


def benzene_minimal(seed=SEED_BASE + 4, b_ee=1.5, b_en=2.0, cc=2.64, ch=2.05):
    """Benzene with a 36-function minimal basis: per carbon C 1s (three most
    diffuse 6-31G C 1s primitives), C 2s and 2p (6-31G SP inner shell); per
    hydrogen 1s (6-31G H inner shell).  MOs: QR of a seeded 36x36 normal
    matrix, MOs 0-20 occupied in both sectors.  Electrons 0-20 spin up, 21-41
    spin down; initial centres as src/systems/benzene.rs:642-655 (six per
    carbon, one per hydrogen), width 0.5 bohr."""
    R = hexagonal_c6h6(cc, ch)
    ao_nuc, ao_l, ao_m, prims = [], [], [], []
    for c in range(6):
        ao_nuc.append(c); ao_l.append(0); ao_m.append(0); prims.append(C_1S[3:])
        ao_nuc.append(c); ao_l.append(0); ao_m.append(0); prims.append(list(zip(C_SP_INNER_EXP, C_SP_INNER_S)))
        for m in range(3):
            ao_nuc.append(c); ao_l.append(1); ao_m.append(m); prims.append(list(zip(C_SP_INNER_EXP, C_SP_INNER_P)))
    for h in range(6):
        ao_nuc.append(6 + h); ao_l.append(0); ao_m.append(0); prims.append(H_INNER)
    Q = seeded_orthonormal(seed, 36)
    init = [i // 6 for i in range(36)] + [6 + h for h in range(6)]
    return SystemSpec(
        name="C6H6-min", spins=[1] * 21 + [-1] * 21, nuc_pos=R, nuc_charge=[6.0] * 6 + [1.0] * 6,
        nuc_species=[0] * 6 + [1] * 6, basis_kind=L.QMC_BASIS_GTO, ao_nuc=ao_nuc, ao_l=ao_l, ao_m=ao_m,
        ao_prims=prims, mo_coef=Q.T.copy(), occ=list(range(21)) * 2, jastrow_kind=L.QMC_JAS_PADE_EEN,
        jas=jastrow3_params(b_ee, b_en), init_nuc=init, init_sigma=0.5)


def _benzene_631g_mos(R):
    """The 21 occupied MOs of BenzeneGTO::build_mo_coefficients
    (src/systems/benzene.rs:247-470) over the 66 AOs in the order of
    ``benzene_gto``: per carbon [1s, 2s in, 2p in (x, y, z), 2s out, 2p out
    (x, y, z)] at 9 n, per hydrogen [1s in, 1s out] at 54 + 2 n.  Core 1s per
    carbon; ring sigma (a1g and the cos/sin e1u pair over 2s and radial 2p);
    one C-H sigma per bond (2s, 2p along C->H, H 1s); pi (a2u, e1g cos/sin over
    2pz); tangential ring sigma (uniform, cos 2t, sin 2t)."""
    C, H = R[:6], R[6:]
    mo = np.zeros((21, 66))
    s6, s3 = 1.0 / math.sqrt(6.0), 1.0 / math.sqrt(3.0)
    ang = [math.pi / 3.0 * n for n in range(6)]
    for n in range(6):                                   # MOs 0-5: carbon cores
        mo[n, 9 * n], mo[n, 9 * n + 1], mo[n, 9 * n + 5] = 0.9943, 0.0234, 0.0020
    for n in range(6):                                   # MOs 6-8: ring sigma from 2s (+ radial 2p)
        mo[6, 9 * n + 1], mo[6, 9 * n + 5] = 0.20 * s6, 0.80 * s6
        for k, f, pm in ((7, math.cos(ang[n]), 0), (8, math.sin(ang[n]), 1)):
            w = f * s3
            mo[k, 9 * n + 1], mo[k, 9 * n + 5] = 0.20 * w, 0.80 * w
            mo[k, 9 * n + 2 + pm], mo[k, 9 * n + 6 + pm] = 0.50 * w, 0.55 * w
    for n in range(6):                                   # MOs 9-14: C-H bonds
        d = (H[n] - C[n]) / np.linalg.norm(H[n] - C[n])
        k = 9 + n
        mo[k, 9 * n + 1], mo[k, 9 * n + 5] = 0.15, 0.30
        for m in range(3):
            mo[k, 9 * n + 2 + m], mo[k, 9 * n + 6 + m] = 0.20 * d[m], 0.55 * d[m]
        mo[k, 54 + 2 * n], mo[k, 54 + 2 * n + 1] = 0.25, 0.15
    for n in range(6):                                   # MOs 15-17: pi
        for k, w in ((15, s6), (16, math.cos(ang[n]) * s3), (17, math.sin(ang[n]) * s3)):
            mo[k, 9 * n + 4], mo[k, 9 * n + 8] = 0.30 * w, 0.70 * w
    for n in range(6):                                   # MOs 18-20: tangential ring sigma
        tx, ty = -math.sin(ang[n]), math.cos(ang[n])
        for k, w in ((18, s6), (19, math.cos(2 * ang[n]) * s3), (20, math.sin(2 * ang[n]) * s3)):
            mo[k, 9 * n + 2], mo[k, 9 * n + 3] = 0.25 * tx * w, 0.25 * ty * w
            mo[k, 9 * n + 6], mo[k, 9 * n + 7] = 0.60 * tx * w, 0.60 * ty * w
    return mo


def benzene_gto(b_ee=1.5, b_en=2.0):
    """BenzeneGTO (src/systems/benzene.rs:48-470): D6h ring with C-C 2.640
    and C-H 2.042 bohr, the 6-31G basis of MethaneGTO on every atom (66 AOs,
    build_631g_basis at benzene.rs:152-245), the hand-built 21-MO table,
    Jastrow3 (a_anti 0.5, a_para 0.25, A = 1, one b_en for both species).
    Electrons 0-20 spin up, 21-41 spin down, both sectors over MOs 0-20;
    initial centres as benzene.rs:642-655."""
    R = hexagonal_c6h6(2.640, 2.042)
    ao_nuc, ao_l, ao_m, prims = [], [], [], []

    def add(n, l, m, p):
        ao_nuc.append(n); ao_l.append(l); ao_m.append(m); prims.append(p)

    for c in range(6):
        add(c, 0, 0, C_1S)
        add(c, 0, 0, list(zip(C_SP_INNER_EXP, C_SP_INNER_S)))
        for m in range(3):
            add(c, 1, m, list(zip(C_SP_INNER_EXP, C_SP_INNER_P)))
        add(c, 0, 0, [(C_SP_OUTER_EXP, 1.0)])
        for m in range(3):
            add(c, 1, m, [(C_SP_OUTER_EXP, 1.0)])
    for h in range(6):
        add(6 + h, 0, 0, H_INNER)
        add(6 + h, 0, 0, [(H_OUTER_EXP, 1.0)])
    init = [i // 6 for i in range(36)] + [6 + h for h in range(6)]
    return SystemSpec(
        name="C6H6-6-31G", spins=[1] * 21 + [-1] * 21, nuc_pos=R, nuc_charge=[6.0] * 6 + [1.0] * 6,
        nuc_species=[0] * 6 + [1] * 6, basis_kind=L.QMC_BASIS_GTO, ao_nuc=ao_nuc, ao_l=ao_l, ao_m=ao_m,
        ao_prims=prims, mo_coef=_benzene_631g_mos(R), occ=list(range(21)) * 2, jastrow_kind=L.QMC_JAS_PADE_EEN,
        jas=jastrow3_params(b_ee, b_en), init_nuc=init, init_sigma=0.5)


def monkhorst_pack_grid(n):
    """Twists of an n x n x n Monkhorst-Pack grid in reduced coordinates
    (src/systems/heg.rs:176-190): theta_s = (2 s - n - 1) / (2 n), s = 1..n,
    generated in i, j, k order."""
    th = [(2.0 * (i + 1.0) - n - 1.0) / (2.0 * n) for i in range(n)]
    return np.array([[tx, ty, tz] for tx in th for ty in th for tz in th]).reshape(-1, 3)


def heg_k_vectors(n, L, twist=None):
    """The n lowest plane waves k + theta (2 pi / L) of a cubic box
    (src/systems/heg.rs:194-232): integer vectors in [-m, m]^3 generated in
    nx, ny, nz order, shifted by the twist and stably sorted by |k + theta|^2,
    m = ceil(2 n^(1/3)) + 2."""
    m = int(math.ceil(n ** (1.0 / 3.0) * 2.0)) + 2
    dk = 2.0 * math.pi / L
    tw = (0.0, 0.0, 0.0) if twist is None else tuple(float(t) for t in twist)
    kt = (tw[0] * dk, tw[1] * dk, tw[2] * dk)
    cand = []
    for nx in range(-m, m + 1):
        for ny in range(-m, m + 1):
            for nz in range(-m, m + 1):
                kx, ky, kz = nx * dk + kt[0], ny * dk + kt[1], nz * dk + kt[2]
                cand.append((kx * kx + ky * ky + kz * kz, kx, ky, kz))
    cand.sort(key=lambda t: t[0])        # Python's sort is stable, like Rust's sort_by
    return np.array([[c[1], c[2], c[3]] for c in cand[:n]])


HEG_FORMS = {"pade": 0, "rpa": 1, "yukawa": 2}


def electron_gas(n_elec=54, rs=4.0, F=7.0, form="rpa", reference_quirks=False, alpha_L=4.0, kmax=6, twist=None):
    """Homogeneous electron gas (src/systems/heg.rs:119-170): box
    L = (4 pi N / 3)^(1/3) r_s, closed-shell plane-wave determinants (N/2 per
    spin, same k set), Jastrow u = A r/(1 + r/F + 0.2 r^2/F^2) (RPA form) with
    the reference's amplitudes A_same = 0.5, A_anti = 0.25, minimum image and
    cutoff at L/2.  With ``reference_quirks`` the Ewald sum and cross term are
    the reference's; otherwise the one-component-plasma Ewald sum with
    alpha = alpha_L / L (alpha_L >= 3.74: real-space images within 5.6/alpha
    < 1.5 L) and |n| <= kmax reciprocal vectors.  The default (4, 6) keeps the
    Ewald energy within 1e-10 Ha of the converged value with 462 vectors.
    ``twist`` (reduced coordinates, heg.rs:116-131) shifts every orbital wave
    vector by theta 2 pi / L; |psi|^2, the drift and E_L are periodic for any
    twist, so the same kernels run twisted boundary conditions."""
    box = (4.0 * math.pi / 3.0 * n_elec) ** (1.0 / 3.0) * rs
    nup = n_elec // 2
    k = heg_k_vectors(nup, box, twist)
    jas = np.zeros(8)
    jas[0] = HEG_FORMS[form]
    jas[2], jas[3] = 0.25, 0.5          # antiparallel, parallel (heg.rs:146-147)
    jas[4], jas[5] = alpha_L, kmax
    quirks = (4 | 8) if reference_quirks else 0
    return SystemSpec(
        name="HEG-%d" % n_elec, spins=[1] * nup + [-1] * (n_elec - nup), nuc_pos=np.zeros((0, 3)), nuc_charge=[],
        basis_kind=L.QMC_BASIS_PW, ao_nuc=[], ao_l=[], ao_m=[], ao_prims=[], mo_coef=k,
        occ=list(range(nup)) + list(range(n_elec - nup)), jastrow_kind=3, jas_F=F, jas=jas, quirks=quirks,
        init_sigma=-1.0, box_L=box)
