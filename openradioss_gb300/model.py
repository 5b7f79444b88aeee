"""Host-side model preparation (the starter's decisions for this path).

Builds, with numpy, the arrays the engine receives from the starter for the
explicit hot path, in the reference's own layouts:

* nodal coordinates ``X(3,NUMNOD)`` / velocities ``V(3,NUMNOD)`` /
  masses ``MS(NUMNOD)``;
* hexa connectivity ``IXS(11,NUMELS)`` = {mat, n1..n8 (1-based), prop,
  user id} (starter/source/elements/solid/solide/sgrtails.F);
* shell connectivity ``IXC(7,NUMELC)`` = {mat, n1..n4, prop, user id};
* material columns ``PM(1:NPROPM)`` and property columns ``GEO(1:NPROPG)``
  holding the entries the path reads (LAW1: hm_read_mat01.F; LAW2:
  hm_read_mat02_jc.F90; solid property: hm_read_prop14.F; shell property:
  hm_read_prop01.F), plus LAW2 ``mat_param%uparam`` / ``iparam``;
* boundary codes (bit 1/2/4 = fixed x/y/z translation, 8/16/32 rotations).

The synthetic meshes are the workloads the benchmark and the tests run: a
structured one-point hexa block (bar impact, large block) and a square crash
box of 4-node shells.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

NPROPM = 128
NPROPG = 256
NUPARAM = 16
NIPARAM = 8


# --------------------------------------------------------------------------
# materials / properties
# --------------------------------------------------------------------------
def _g_bulk(young, nu):
    if nu == 0.5:
        nu = 0.499  # ZEP499 (hm_read_mat01.F)
    g = young / (2.0 * (1.0 + nu))
    c1 = young / (3.0 * (1.0 - 2.0 * nu))
    return g, c1


def _plane_stress(pm, young, nu, rho):
    """PM(24) = E/(1-nu^2), PM(25) = nu*PM(24), PM(27) = sqrt(E/rho): the
    plane-stress modulus and sound speed the shell path reads
    (hm_read_mat02_jc.F90:151-160)."""
    a11 = young / (1.0 - nu ** 2)
    pm[23] = a11
    pm[24] = nu * a11
    pm[26] = math.sqrt(young / max(rho, 1e-20))


def law1(rho, young, nu):
    """/MAT/ELAST (LAW1): PM(1)=rho, PM(20)=E, PM(21)=nu, PM(22)=G, PM(32)=C1."""
    pm = np.zeros(NPROPM)
    g, c1 = _g_bulk(young, nu)
    pm[0] = rho
    pm[19] = young
    pm[20] = nu
    pm[21] = g
    pm[31] = c1
    _plane_stress(pm, young, nu, rho)
    pm[88] = rho  # PM(89) = RHO0
    return dict(mtn=1, pm=pm, uparam=np.zeros(NUPARAM), iparam=np.zeros(NIPARAM, np.int32))


def law2(rho, young, nu, a, b, n, c=0.0, eps0=1.0, epsmax=0.0, sigmax=0.0,
         m_exp=0.0, vp=0, icc=0, fcut=0.0, fisokin=0.0, rhocp=0.0, tref=0.0, tmelt=0.0):
    """/MAT/PLAS_JOHNS (LAW2, Johnson-Cook) with the reader's defaults
    (starter/source/materials/mat/mat002/hm_read_mat02_jc.F90:100-200,
    249-251, 329-349): FISOKIN in uparam(8), the thermal parameters in
    PM(69) = rho Cp, PM(79) = T_r (300 when not positive), PM(80) = T_melt
    (1e20 when 0)."""
    pm = np.zeros(NPROPM)
    g, bulk = _g_bulk(young, nu)
    if n == 0.0:
        n = 1.0
    if epsmax == 0.0:
        epsmax = 1e20
    if sigmax == 0.0:
        sigmax = 1e20
    if icc == 0:
        icc = 1
    if vp == 0:
        vp = 2
    israte = 1
    if c == 0.0:
        eps0 = 1.0
        israte = 0
    if vp == 1:
        fcut = 10000.0
    asrate = 1e20 if fcut == 0.0 else 2.0 * math.pi * fcut
    if m_exp == 0.0:
        m_exp = 1.0
    pm[0] = rho
    pm[19] = young
    pm[20] = nu
    pm[21] = g
    pm[31] = bulk
    _plane_stress(pm, young, nu, rho)
    pm[37], pm[38], pm[39] = a, b, n
    pm[88] = rho
    if tref <= 0.0:
        tref = 300.0
    if tmelt == 0.0:
        tmelt = 1e20
    pm[68], pm[78], pm[79] = rhocp, tref, tmelt
    up = np.zeros(NUPARAM)
    up[:10] = [a, b, n, epsmax, sigmax, c, eps0, fisokin, asrate, m_exp]
    ip = np.zeros(NIPARAM, np.int32)
    ip[:4] = [0, icc, vp, israte]
    return dict(mtn=2, pm=pm, uparam=up, iparam=ip)


def solid_prop(qa=1.1, qb=0.05, qh=0.1, dn1=0.0, dn2=0.0):
    """/PROP/SOLID Isolid=1, Iframe=1 (JCVT=0), Ismstr=4: GEO(13)=QH,
    GEO(14)=QA, GEO(15)=QB, GEO(16..17) numerical damping."""
    geo = np.zeros(NPROPG)
    geo[12], geo[13], geo[14], geo[15], geo[16] = qh, qa, qb, dn1, dn2
    return geo


def shell_prop(thk, hm=0.01, hf=0.01, hr=0.01, dm=0.0, iplas=1):
    """/PROP/SHELL, Ishell=1 (Belytschko-Tsay, viscous/elastic hourglass),
    Ismstr=4, Ithick=1, with the reader's defaults
    (starter/source/properties/shell/hm_read_prop01.F:200-330):
    GEO(1)=thickness, GEO(13..15)=hm, hf, hr (default 0.01), GEO(16)=dm,
    GEO(37)=Ishear=0, GEO(38)=shear factor 5/6, GEO(39)=Iplas."""
    geo = np.zeros(NPROPG)
    geo[0] = thk
    geo[12], geo[13], geo[14], geo[15] = hm, hf, hr, dm
    geo[36] = 0.0
    geo[37] = 5.0 / 6.0
    geo[38] = float(iplas)
    return geo


# --------------------------------------------------------------------------
# meshes
# --------------------------------------------------------------------------
def hexa_volumes(X, ixs):
    """SDERI3 determinant (sderi3.F) of every hexa, FP64, vectorised."""
    n = ixs[1:9].T - 1
    x, y, z = X[0][n], X[1][n], X[2][n]
    d = lambda a, i, j: a[:, i] - a[:, j]
    x17, x28, x35, x46 = d(x, 6, 0), d(x, 7, 1), d(x, 4, 2), d(x, 5, 3)
    y17, y28, y35, y46 = d(y, 6, 0), d(y, 7, 1), d(y, 4, 2), d(y, 5, 3)
    z17, z28, z35, z46 = d(z, 6, 0), d(z, 7, 1), d(z, 4, 2), d(z, 5, 3)
    j1, j2, j3 = x17 + x28 - x35 - x46, y17 + y28 - y35 - y46, z17 + z28 - z35 - z46
    j4, j5, j6 = (x17 + x46) + (x28 + x35), (y17 + y46) + (y28 + y35), (z17 + z46) + (z28 + z35)
    j7, j8, j9 = (x17 + x46) - (x28 + x35), (y17 + y46) - (y28 + y35), (z17 + z46) - (z28 + z35)
    return (1.0 / 64.0) * (j1 * (j5 * j9 - j6 * j8) + j2 * (j6 * j7 - j4 * j9) + j3 * (j4 * j8 - j5 * j7))


@dataclass
class HexaGroupSpec:
    ixs: np.ndarray            # (11, nel) int32
    mat: dict
    geo: np.ndarray
    jcvt: int = 0              # 0: Iframe=1 (Jaumann), 1: co-rotational frame


@dataclass
class ShellGroupSpec:
    ixc: np.ndarray            # (7, nel) int32
    mat: dict
    geo: np.ndarray
    thk: np.ndarray            # (nel,)
    npt: int = 5
    ithk: int = 1              # 1: current thickness, 0: initial thickness
    ismstr: int = 2


@dataclass
class Model:
    """A deck for the hot path: nodes, element groups, conditions."""
    name: str
    X: np.ndarray              # (3, numnod) float64
    V: np.ndarray              # (3, numnod)
    MS: np.ndarray             # (numnod,)
    icodt: np.ndarray          # (numnod,) int32
    hexa: list = field(default_factory=list)
    shells: list = field(default_factory=list)
    IN: np.ndarray | None = None
    rwalls: list = field(default_factory=list)  # (p0[3], n[3], dsearch)
    # rigid links (engine /VEL/TRA|ROT): (1-based nodes, ic, icr), direction
    # bits 4 = x, 2 = y, 1 = z
    rlinks: list = field(default_factory=list)
    # rigid bodies (/RBODY, after the starter's set-up, rbody_init):
    # (1-based main node, 1-based secondary nodes, principal axes as rows
    # (3, 3), principal inertia (3,))
    rbodies: list = field(default_factory=list)
    # concentrated loads (/CLOAD): (1-based node, direction 0..5, abscissa
    # scale, ordinate scale, curve abscissae, curve ordinates)
    cloads: list = field(default_factory=list)
    # rigid-material bodies (/MAT/RIGID, LAW13, the starter's RIGID_MAT):
    # (1-based secondary nodes, centre of mass (3,), mass, principal axes as
    # rows (3, 3), principal inertia (3,)) -- oracle only, like rbodies
    rmats: list = field(default_factory=list)
    # imposed velocities (/IMPVEL): (1-based node, direction 0..2, 1/abscissa
    # scale, ordinate scale, start, stop, curve abscissae, curve ordinates)
    # -- oracle only
    impvels: list = field(default_factory=list)
    ishfram: int = 0           # local shell frame: 0 symmetric, 2 /SHFRA/V4
    nodal_dt: tuple | None = None  # /DT/NODA: (DTFAC1(11), DTMIN1(11))
    # /DT time-step actions {kind: (IDTMIN, DTMIN1)}: 3 shells (1/5 stop,
    # 2 delete), 11 nodal step (3/8 mass scaling, else stop)
    dtmin_actions: dict = field(default_factory=dict)
    dtfac_solid: float = 0.9
    dtfac_shell: float = 0.9
    dtmx: float = 1e30
    dt2old: float = 1e30

    @property
    def numnod(self):
        return self.X.shape[1]

    @property
    def numels(self):
        return sum(g.ixs.shape[1] for g in self.hexa)

    @property
    def numelc(self):
        return sum(g.ixc.shape[1] for g in self.shells)


def hexa_block(nx, ny, nz, h, origin=(0.0, 0.0, 0.0)):
    """Structured block of nx*ny*nz one-point hexas of edge h.  Node order
    x fastest; element nodes 1-4 on the lower z face counter-clockwise,
    5-8 above (the reference's brick numbering)."""
    ix = np.arange(nx + 1)
    iy = np.arange(ny + 1)
    iz = np.arange(nz + 1)
    gz, gy, gx = np.meshgrid(iz, iy, ix, indexing="ij")
    X = np.stack([origin[0] + h * gx.ravel(), origin[1] + h * gy.ravel(),
                  origin[2] + h * gz.ravel()]).astype(np.float64)
    nid = lambda i, j, k: (k * (ny + 1) + j) * (nx + 1) + i
    ez, ey, ex = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    ex, ey, ez = ex.ravel(), ey.ravel(), ez.ravel()
    conn = np.stack([
        nid(ex, ey, ez), nid(ex + 1, ey, ez), nid(ex + 1, ey + 1, ez), nid(ex, ey + 1, ez),
        nid(ex, ey, ez + 1), nid(ex + 1, ey, ez + 1), nid(ex + 1, ey + 1, ez + 1), nid(ex, ey + 1, ez + 1),
    ]).astype(np.int32)
    nel = conn.shape[1]
    ixs = np.zeros((11, nel), np.int32)
    ixs[0] = 1
    ixs[1:9] = conn + 1
    ixs[9] = 1
    ixs[10] = np.arange(1, nel + 1, dtype=np.int32)
    return X, ixs


def lumped_mass_hexa(X, ixs, rho, ms=None):
    """SMASS3 (starter/source/elements/solid/solide/smass3.F:92): each node
    receives rho*V/8 from every hexa, accumulated in element order."""
    numnod = X.shape[1]
    if ms is None:
        ms = np.zeros(numnod)
    vol = hexa_volumes(X, ixs)
    m8 = rho * vol * 0.125
    for k in range(8):
        np.add.at(ms, ixs[1 + k] - 1, m8)
    return ms


def bar_impact(n=20, h=0.005, v0=10.0, rho=7850.0, young=210e9, nu=0.3,
               law="law1"):
    """Steel bar impact: n^3 one-point hexas, edge h, LAW1 elastic, viscous
    hourglass, the z=0 face fixed, every other node moving at v0 towards it
    (along the face normal)."""
    X, ixs = hexa_block(n, n, n, h)
    mat = law1(rho, young, nu) if law == "law1" else law2(
        rho, young, nu, 350e6, 275e6, 0.36, c=0.022, eps0=1.0)
    ms = lumped_mass_hexa(X, ixs, rho)
    icodt = np.zeros(X.shape[1], np.int32)
    fixed = X[2] == 0.0
    icodt[fixed] = 7
    V = np.zeros_like(X)
    V[2, ~fixed] = -v0
    return Model("bar_impact_%d" % n, X, V, ms, icodt,
                 hexa=[HexaGroupSpec(ixs, mat, solid_prop())])


def large_block(n=128, h=0.005, vmean=20.0, vstd=0.5, seed=1, rho=7850.0,
                young=210e9, nu=0.3, law="law2"):
    """Large hexa block with Johnson-Cook: n^3 one-point hexas, seeded
    initial velocity 20 m/s + N(0, 0.5) per node component."""
    X, ixs = hexa_block(n, n, n, h)
    mat = law2(rho, young, nu, 350e6, 275e6, 0.36, c=0.022, eps0=1.0) \
        if law == "law2" else law1(rho, young, nu)
    ms = lumped_mass_hexa(X, ixs, rho)
    rng = np.random.default_rng(seed)
    V = rng.normal(0.0, vstd, size=X.shape)
    V[2] += -vmean
    icodt = np.zeros(X.shape[1], np.int32)
    icodt[X[2] == 0.0] = 7
    V[:, X[2] == 0.0] = 0.0
    return Model("large_block_%d" % n, X, V, ms, icodt,
                 hexa=[HexaGroupSpec(ixs, mat, solid_prop())])


def shell_mass_inertia(X, ixc, thk, rho, ms=None, inr=None):
    """Nodal mass and rotational inertia of 4-node shells
    (starter/source/elements/shell/coque/cinmas.F): each node receives
    EMS = rho*t*A/4 and EMS*(A/9 + t^2/12) (FAC = 9 for Ishell < 11)."""
    numnod = X.shape[1]
    ms = np.zeros(numnod) if ms is None else ms
    inr = np.zeros(numnod) if inr is None else inr
    n = ixc[1:5] - 1
    p = [X[:, n[k]] for k in range(4)]
    # area of the quadrilateral: half the norm of the diagonals' cross product
    d13, d24 = p[2] - p[0], p[3] - p[1]
    area = 0.5 * np.linalg.norm(np.cross(d13.T, d24.T), axis=1)
    ems = rho * thk * area * 0.25
    xi = ems * (area / 9.0 + thk * thk / 12.0)
    for k in range(4):
        np.add.at(ms, n[k], ems)
        np.add.at(inr, n[k], xi)
    return ms, inr


def crash_box(n_side=77, n_len=390, side=0.060, length=0.300, thk=1.2e-3,
              v0=15.0, seed=0, rho=7850.0, young=210e9, nu=0.3,
              a=350e6, b=275e6, n=0.36, c=0.022, gap=1e-4, npt=5, vpert=0.0):
    """Square crash box of Belytschko-Tsay shells: a tube of square section
    (side x side) and the given length along z, n_side elements per face
    across and n_len along (4*n_side*n_len shells), thickness thk, NPT
    through-thickness points, Johnson-Cook LAW2.  Nodes get a seeded
    imperfection U[-0.1 t, 0.1 t] along their face normal; the box moves at
    v0 towards a fixed planar rigid wall just below its lower end.  vpert > 0
    adds a seeded N(0, vpert) velocity to every node (deformation from the
    first cycle on)."""
    per = 4 * n_side
    s = np.linspace(0.0, 4.0 * side, per + 1)[:-1]
    face = (s // side).astype(int)
    u = s - face * side
    h = side / 2.0
    xs = np.where(face == 0, -h + u, np.where(face == 1, h, np.where(face == 2, h - u, -h)))
    ys = np.where(face == 0, -h, np.where(face == 1, -h + u, np.where(face == 2, h, h - u)))
    nxn = np.where(face == 0, 0.0, np.where(face == 1, 1.0, np.where(face == 2, 0.0, -1.0)))
    nyn = np.where(face == 0, -1.0, np.where(face == 1, 0.0, np.where(face == 2, 1.0, 0.0)))
    corner = (u == 0.0)
    zs = np.linspace(0.0, length, n_len + 1)
    numnod = per * (n_len + 1)
    X = np.zeros((3, numnod))
    X[0] = np.tile(xs, n_len + 1)
    X[1] = np.tile(ys, n_len + 1)
    X[2] = np.repeat(zs, per)
    rng = np.random.default_rng(seed)
    amp = rng.uniform(-0.1 * thk, 0.1 * thk, size=numnod)
    cn = np.tile(corner, n_len + 1)
    amp[cn] = 0.0
    X[0] += amp * np.tile(nxn, n_len + 1)
    X[1] += amp * np.tile(nyn, n_len + 1)
    nid = lambda i, j: j * per + (i % per)
    ii, jj = np.meshgrid(np.arange(per), np.arange(n_len), indexing="xy")
    ii, jj = ii.ravel(), jj.ravel()
    conn = np.stack([nid(ii, jj), nid(ii + 1, jj), nid(ii + 1, jj + 1), nid(ii, jj + 1)])
    nel = conn.shape[1]
    ixc = np.zeros((7, nel), np.int32)
    ixc[0] = 1
    ixc[1:5] = conn + 1
    ixc[5] = 1
    ixc[6] = np.arange(1, nel + 1, dtype=np.int32)
    t = np.full(nel, thk)
    mat = law2(rho, young, nu, a, b, n, c=c, eps0=1.0)
    ms, inr = shell_mass_inertia(X, ixc, t, rho)
    V = np.zeros_like(X)
    V[2] = -v0
    if vpert > 0.0:
        V += rng.normal(0.0, vpert, size=V.shape)
    icodt = np.zeros(numnod, np.int32)
    m = Model("crash_box_%d" % nel, X, V, ms, icodt,
              shells=[ShellGroupSpec(ixc, mat, shell_prop(thk), t, npt)], IN=inr)
    m.rwalls = [((0.0, 0.0, -gap), (0.0, 0.0, 1.0), 2.0 * length)]
    return m


def crash_box_variant(i, seed0=100):
    """Variant i of the batched crash-box sweep: element count U[5k, 60k],
    section U[40, 80] mm, length U[200, 400] mm, thickness U[0.8, 2.0] mm,
    Johnson-Cook A U[250, 450] MPa, impact speed U[8, 20] m/s, all drawn from
    the seeded generator of seed seed0 + i (which also seeds the
    imperfections).  The element edge follows from the element count."""
    rng = np.random.default_rng(seed0 + i)
    nel = rng.uniform(5e3, 6e4)
    side = rng.uniform(40.0, 80.0) * 1e-3
    length = rng.uniform(200.0, 400.0) * 1e-3
    thk = rng.uniform(0.8, 2.0) * 1e-3
    a = rng.uniform(250.0, 450.0) * 1e6
    v0 = rng.uniform(8.0, 20.0)
    h = np.sqrt(4.0 * side * length / nel)
    ns = max(2, int(round(side / h)))
    nl = max(2, int(round(length / h)))
    m = crash_box(n_side=ns, n_len=nl, side=side, length=length, thk=thk, v0=v0,
                  seed=seed0 + i, a=a)
    m.name = "crash_box_variant_%d" % i
    return m


def crash_box_sweep(n=64, seed0=100):
    """The batched sweep: n crash-box variants (seeds seed0 .. seed0+n-1)."""
    return [crash_box_variant(i, seed0) for i in range(n)]


def hexa_impact_block(nel, h=0.005, v0=10.0, vstd=0.5, seed=0, law="law2", a=350e6):
    """Hexa impact block of about nel one-point hexas: a bar of square
    section (nx = ny, nz = 2 nx) with its z=0 face fixed and a seeded velocity
    field v0 + N(0, vstd) towards that face."""
    nx = max(2, int(round((nel / 2.0) ** (1.0 / 3.0))))
    nz = max(2, int(round(nel / (nx * nx))))
    X, ixs = hexa_block(nx, nx, nz, h)
    mat = law2(7850.0, 210e9, 0.3, a, 275e6, 0.36, c=0.022, eps0=1.0) \
        if law == "law2" else law1(7850.0, 210e9, 0.3)
    ms = lumped_mass_hexa(X, ixs, 7850.0)
    rng = np.random.default_rng(seed)
    V = rng.normal(0.0, vstd, size=X.shape)
    V[2] += -v0
    icodt = np.zeros(X.shape[1], np.int32)
    fixed = X[2] == 0.0
    icodt[fixed] = 7
    V[:, fixed] = 0.0
    return Model("hexa_impact_%d" % ixs.shape[1], X, V, ms, icodt,
                 hexa=[HexaGroupSpec(ixs, mat, solid_prop())])


def serving_job(k, seed=7):
    """Job k of the serving stream (seeded): a 50/50 draw between a shell
    crash box of U[2k, 150k] elements and a hexa impact block of U[2k, 200k]
    elements, U[2000, 20000] cycles, LAW1 or LAW2 (hexa blocks) / LAW2
    (shells) with A U[250, 450] MPa and speeds U[8, 20] m/s.  Returns
    (model, ncycles)."""
    rng = np.random.default_rng([seed, k])
    shell = rng.uniform() < 0.5
    ncyc = int(rng.integers(2000, 20001))
    a = rng.uniform(250.0, 450.0) * 1e6
    v0 = rng.uniform(8.0, 20.0)
    if shell:
        nel = rng.uniform(2e3, 1.5e5)
        side = rng.uniform(40.0, 80.0) * 1e-3
        length = rng.uniform(200.0, 400.0) * 1e-3
        thk = rng.uniform(0.8, 2.0) * 1e-3
        h = np.sqrt(4.0 * side * length / nel)
        m = crash_box(n_side=max(2, int(round(side / h))),
                      n_len=max(2, int(round(length / h))), side=side, length=length,
                      thk=thk, v0=v0, seed=1000 + k, a=a)
    else:
        nel = rng.uniform(2e3, 2e5)
        law = "law1" if rng.uniform() < 0.5 else "law2"
        m = hexa_impact_block(nel, v0=v0, seed=1000 + k, law=law, a=a)
    m.name = "job_%d" % k
    return m, ncyc


# --------------------------------------------------------------------------
# decks read into arrays
# --------------------------------------------------------------------------
def _code_bits(digits, base):
    """'101' (x, y, z flags of a /BCS card) -> bits base*{1, 2, 4}."""
    return sum(base * (1 << k) for k in range(3) if digits[k] == "1")


def model_from_deck(d, name="deck", with_links=True):
    """Model of a shell deck held as arrays (the layout written by
    tests/golden/make_cra2.py: nodes, /SHELL parts, /MAT/PLAS_JOHNS,
    /PROP/SHELL, /DEF_SHELL, /SHFRA/V4, /BCS, /INIVEL/TRA, /ADMAS/0, engine
    /VEL/TRA/XYZ links), with the starter's decisions for it:

    * properties: Ishell 0 -> the /DEF_SHELL value, else 1; Ismstr 0 -> 2;
      Ithick / Iplas 0 -> the /DEF_SHELL value; shear factor 0 -> 5/6; N = 0
      with LAW2 -> 3 integration points
      (starter/source/properties/shell/hm_read_prop01.F:177-273,
      starter/source/elements/shell/coque/cgrtails.F:800-811);
    * masses: cinmas lumping of every shell plus the /ADMAS masses;
    * /SHFRA/V4 -> ISHFRAM = 2 (starter/source/starter/contrl.F:495-498).

    Node and element ids must run 1..n (they do in the decks used here).
    """
    node_id = np.asarray(d["node_id"])
    if not np.array_equal(node_id, np.arange(1, len(node_id) + 1)):
        raise ValueError("node ids must be 1..numnod")
    X = np.ascontiguousarray(np.asarray(d["X"], np.float64).T)
    numnod = X.shape[1]
    mcols = [str(c) for c in d["mat_columns"]]
    pcols = [str(c) for c in d["prop_columns"]]
    mats = {int(r[0]): dict(zip(mcols, r)) for r in np.asarray(d["mat"])}
    props = {int(r[0]): dict(zip(pcols, r)) for r in np.asarray(d["prop"])}
    ds = [int(v) for v in d["def_shell"]]  # ISHELL ISMSTR ITHICK IPLAS ISTRAIN ISH3N IDRIL
    ms = np.zeros(numnod)
    inr = np.zeros(numnod)
    shells = []
    sid = np.asarray(d["shell_id"])
    spart = np.asarray(d["shell_part"])
    snodes = np.asarray(d["shell_nodes"])
    for p, mid, pid in zip(d["part_id"], d["part_mat"], d["part_prop"]):
        sel = np.nonzero(spart == p)[0]
        mt, pr = mats[int(mid)], props[int(pid)]
        ihbe = int(pr["Ishell"]) or ds[0] or 1
        if ihbe != 1:
            raise ValueError("only Ishell = 1 shells are supported")
        ismstr = int(pr["Ismstr"]) or ds[1] or 2
        ithk = int(pr["Ithick"]) or ds[2]
        ipla = int(pr["Iplas"]) or ds[3]
        npt = int(pr["N"]) or 3
        thick = float(pr["Thick"])
        mat = law2(mt["rho"], mt["E"], mt["nu"], mt["a"], mt["b"], mt["n"], c=mt["c"],
                   eps0=mt["eps0"], epsmax=mt["epsmax"], sigmax=mt["sigmax"], m_exp=mt["m"],
                   icc=int(mt["ICC"]), fcut=mt["Fcut"])
        geo = shell_prop(thick, hm=pr["hm"] or 0.01, hf=pr["hf"] or 0.01, hr=pr["hr"] or 0.01,
                         dm=pr["dm"], iplas=ipla)
        if pr["Ashear"]:
            geo[37] = pr["Ashear"]
        ixc = np.zeros((7, len(sel)), np.int32)
        ixc[0] = int(mid)
        ixc[1:5] = snodes[sel].T
        ixc[5] = int(pid)
        ixc[6] = sid[sel]
        t = np.full(len(sel), thick)
        shell_mass_inertia(X, ixc, t, mt["rho"], ms, inr)
        shells.append(ShellGroupSpec(ixc, mat, geo, t, npt, ithk=ithk, ismstr=ismstr))
    ms[np.asarray(d["admas_nodes"]) - 1] += float(d["admas"])
    icodt = np.zeros(numnod, np.int32)
    off = np.asarray(d["bcs_offsets"])
    bn = np.asarray(d["bcs_nodes"])
    for k, (tra, rot) in enumerate(zip(d["bcs_tra"], d["bcs_rot"])):
        code = _code_bits(str(tra), 1) | _code_bits(str(rot), 8)
        icodt[bn[off[k]:off[k + 1]] - 1] |= code
    V = np.zeros_like(X)
    V[:, np.asarray(d["inivel_nodes"]) - 1] = np.asarray(d["inivel"], np.float64)[:, None]
    m = Model(name, X, V, ms, icodt, shells=shells, IN=inr)
    if with_links and len(d["rlink_nodes"]):
        m.rlinks = [(np.asarray(d["rlink_nodes"], np.int32), 7, 0)]
    m.ishfram = 2 if int(d["shfra_v4"]) else 0
    return m


def rbody_init(X, MS, IN, main, nodes, ispher=2):
    """The starter's rigid-body set-up INIRBY
    (starter/source/constraints/general/rbody/inirby.F) for a body without
    added mass or inertia, skew or sensor, centre-of-mass flag ICOG = 1:
    the main node (1-based) moves to the centre of mass of itself (a zero
    mass counts as 1e-20) and the secondary nodes (1-based); the inertia
    tensor about it collects the main node's shifted mass, the secondary
    masses and their nodal inertia; its principal values below 1e-3 of the
    largest gain 0.1 of the largest (ISPHER = 2, the reader's default);
    MS(main) becomes the body mass and IN(main) the smallest principal
    inertia.  X, MS, IN are updated in place.  Returns the principal axes as
    rows (right-handed) and the principal inertia."""
    m = int(main) - 1
    sec = np.asarray(nodes, np.int64) - 1
    ms_loc, in_loc = MS[sec].copy(), IN[sec].copy()
    if MS[m] == 0.0:
        MS[m] = 1e-20
    J = np.eye(3) * IN[m]
    xmg = MS[m]
    xg = X[:, m].copy()
    masrb = MS[m] + ms_loc.sum()
    X[:, m] = (X[:, m] * MS[m] + (X[:, sec] * ms_loc).sum(axis=1)) / masrb
    r = xg - X[:, m]
    J += xmg * (np.dot(r, r) * np.eye(3) - np.outer(r, r))
    for k in range(len(sec)):
        r = X[:, sec[k]] - X[:, m]
        J += in_loc[k] * np.eye(3) + ms_loc[k] * (np.dot(r, r) * np.eye(3) - np.outer(r, r))
    w, v = np.linalg.eigh(J)
    if ispher == 2 and w.min() <= 1e-3 * w.max():
        w = np.where(w / w.max() < 1e-3, w + 0.1 * w.max(), w)
    axes = v.T.copy()
    if np.linalg.det(axes) < 0:
        axes[2] = -axes[2]
    MS[m] = masrb
    IN[m] = w.min()
    return axes, w, J


def hexa_model_from_deck(d, name="deck"):
    """Model of a hexa deck held as arrays (the layout written by
    tests/golden/make_h101.py: nodes, /BRICK parts, /MAT/ELAST, /PROP/SOLID,
    /DEF_SOLID, /BCS, /FUNCT + /CLOAD, /RBODY), with the starter's decisions
    for it:

    * properties (starter/source/properties/solid/hm_read_prop14.F:276-288):
      Isolid 0 -> the /DEF_SOLID value; Iframe 0 -> the /DEF_SOLID value, and
      Iframe 2 is the co-rotational frame (JCVT = 1 in the engine); Ismstr 0
      -> 4; qa, qb, h 0 -> 1.1, 0.05, 0.1;
    * masses: SMASS3 lumping rho V / 8 of every brick;
    * rigid bodies: rbody_init (INIRBY).

    Node ids are mapped to 1-based indices in the order of the /NODE card;
    elements keep their user ids.  One hexa group per part, in part order.
    """
    node_id = np.asarray(d["node_id"])
    index = {int(n): k + 1 for k, n in enumerate(node_id)}
    to_idx = np.vectorize(lambda n: index[int(n)], otypes=[np.int32])
    X = np.ascontiguousarray(np.asarray(d["X"], np.float64).T)
    numnod = X.shape[1]
    mats = {int(r[0]): r for r in np.asarray(d["mat"])}
    pcols = [str(c) for c in d["prop_columns"]]
    props = {int(r[0]): dict(zip(pcols, r)) for r in np.asarray(d["prop"])}
    isolid_d, ismstr_d, _, iframe_d = (int(v) for v in d["def_solid"])
    ms = np.zeros(numnod)
    groups = []
    bid, bpart, bnodes = (np.asarray(d[k]) for k in ("brick_id", "brick_part", "brick_nodes"))
    for p, mid, pid in zip(d["part_id"], d["part_mat"], d["part_prop"]):
        sel = np.nonzero(bpart == p)[0]
        _, rho, young, nu = mats[int(mid)]
        pr = props[int(pid)]
        isolid = int(pr["Isolid"]) or isolid_d or 1
        iframe = int(pr["Iframe"]) or iframe_d
        ismstr = int(pr["Ismstr"]) or ismstr_d or 4
        if isolid != 1 or ismstr != 4 or iframe not in (1, 2):
            raise ValueError("only Isolid = 1, Ismstr = 4 bricks are supported")
        ixs = np.zeros((11, len(sel)), np.int32)
        ixs[0] = int(mid)
        ixs[1:9] = to_idx(bnodes[sel]).T
        ixs[9] = int(pid)
        ixs[10] = bid[sel]
        lumped_mass_hexa(X, ixs, rho, ms)
        geo = solid_prop(qa=pr["qa"] or 1.1, qb=pr["qb"] or 0.05, qh=pr["h"] or 0.1)
        groups.append(HexaGroupSpec(ixs, law1(rho, young, nu), geo, jcvt=iframe - 1))
    icodt = np.zeros(numnod, np.int32)
    off = np.asarray(d["bcs_offsets"])
    bn = to_idx(np.asarray(d["bcs_nodes"]))
    for k, (tra, rot) in enumerate(zip(d["bcs_tra"], d["bcs_rot"])):
        icodt[bn[off[k]:off[k + 1]] - 1] |= _code_bits(str(tra), 1) | _code_bits(str(rot), 8)
    inr = np.zeros(numnod)
    rbodies = []
    off = np.asarray(d["rbody_offsets"])
    rn = np.asarray(d["rbody_nodes"])
    for k, main in enumerate(d["rbody_main"]):
        nodes = to_idx(rn[off[k]:off[k + 1]])
        axes, inertia, _ = rbody_init(X, ms, inr, index[int(main)], nodes)
        rbodies.append((index[int(main)], nodes, axes, inertia))
    fx, fy = np.asarray(d["funct1"], np.float64).T
    fcx, fcy = (float(v) for v in d["cload_scale"])
    cloads = [(index[int(n)], int(d["cload_dir"]), fcx, fcy, fx, fy) for n in d["cload_nodes"]]
    m = Model(name, X, np.zeros_like(X), ms, icodt, hexa=groups, IN=inr)
    m.rbodies = rbodies
    m.cloads = cloads
    return m


def rigid_mat_init(X, MS, IN, nodes):
    """The starter's RIGID_MAT (starter/source/materials/mat/mat019/
    rigid_mat.F) for one rigid-material body of 1-based secondary nodes: mass
    = the nodes' masses, centre of mass, the inertia tensor about it (nodal
    inertia plus the point masses), its principal inertia and axes (rows,
    right-handed).  Returns (centre, mass, axes, inertia)."""
    sec = np.asarray(nodes, np.int64) - 1
    ms = MS[sec]
    mass = float(ms.sum())
    xg = (X[:, sec] * ms).sum(axis=1) / mass
    J = np.zeros((3, 3))
    for k, n in enumerate(sec):
        r = X[:, n] - xg
        J += IN[n] * np.eye(3) + ms[k] * (np.dot(r, r) * np.eye(3) - np.outer(r, r))
    w, v = np.linalg.eigh(J)
    axes = v.T.copy()
    if np.linalg.det(axes) < 0:
        axes[2] = -axes[2]
    return xg, mass, axes, w


def rigid_material_bodies(ixs_rigid):
    """ININODE_RM (starter/source/materials/mat/mat019/ininode_rm.F): the
    rigid-material bricks (1-based node columns, (8, n)) grouped into bodies
    of bricks connected through shared nodes; each body's nodes, sorted."""
    n = ixs_rigid.shape[1]
    parent = list(range(n))

    def root(i):
        while parent[i] != i:
            parent[i] = parent[parent[i]]
            i = parent[i]
        return i
    owner = {}
    for e in range(n):
        for nd in ixs_rigid[:, e]:
            nd = int(nd)
            if nd in owner:
                a, b = root(owner[nd]), root(e)
                if a != b:
                    parent[max(a, b)] = min(a, b)
            else:
                owner[nd] = e
    groups = {}
    for e in range(n):
        groups.setdefault(root(e), set()).update(int(v) for v in ixs_rigid[:, e])
    return [np.array(sorted(groups[k]), np.int32) for k in sorted(groups)]


def rigid_jc_model_from_deck(d, name="deck"):
    """Model of a hexa deck with Johnson-Cook and rigid-material parts held
    as arrays (the layout written by tests/golden/make_loi13.py: nodes,
    /BRICK parts, /MAT/PLAS_JOHNS, /MAT/RIGID, /PROP/SOLID, /BCS, /IMPVEL +
    /FUNCT), with the starter's decisions for it:

    * the Johnson-Cook part: Isolid = 1, Ismstr 0 -> 4, Iframe 2 -> the
      co-rotational frame (JCVT = 1); LAW2 with the reader's defaults;
    * masses: SMASS3 lumping rho V / 8 of every brick, rigid ones included;
    * the rigid-material parts (LAW13) run no element (FORINT skips them):
      their bricks form rigid-material bodies (ININODE_RM), set up by
      rigid_mat_init (RIGID_MAT);
    * /IMPVEL: abscissa scale 0 -> 1 (stored inverted), ordinate scale 0 ->
      1, stop time 0 -> infinity.

    Node ids are mapped to 1-based indices in the order of the /NODE card;
    elements keep their user ids."""
    node_id = np.asarray(d["node_id"])
    index = {int(n): k + 1 for k, n in enumerate(node_id)}
    to_idx = np.vectorize(lambda n: index[int(n)], otypes=[np.int32])
    X = np.ascontiguousarray(np.asarray(d["X"], np.float64).T)
    numnod = X.shape[1]
    jc = dict(zip([str(c) for c in d["mat_jc_columns"]], np.asarray(d["mat_jc"])))
    rigid = {int(r[0]): r for r in np.asarray(d["mat_rigid"])}
    pr = dict(zip([str(c) for c in d["prop_columns"]], np.asarray(d["prop"])))
    if int(pr["Isolid"]) not in (0, 1) or int(pr["Ismstr"]) not in (0, 4) or \
            int(pr["Iframe"]) not in (1, 2):
        raise ValueError("only Isolid = 1, Ismstr = 4 bricks are supported")
    ms = np.zeros(numnod)
    groups, rigid_cols = [], []
    bid, bpart, bnodes = (np.asarray(d[k]) for k in ("brick_id", "brick_part", "brick_nodes"))
    for p, mid, pid in zip(d["part_id"], d["part_mat"], d["part_prop"]):
        sel = np.nonzero(bpart == p)[0]
        ixs = np.zeros((11, len(sel)), np.int32)
        ixs[0] = int(mid)
        ixs[1:9] = to_idx(bnodes[sel]).T
        ixs[9] = int(pid)
        ixs[10] = bid[sel]
        if int(mid) in rigid:
            lumped_mass_hexa(X, ixs, float(rigid[int(mid)][1]), ms)
            rigid_cols.append(ixs[1:9])
            continue
        if int(mid) != int(jc["id"]):
            raise ValueError("unexpected material %d" % int(mid))
        lumped_mass_hexa(X, ixs, float(jc["rho"]), ms)
        mat = law2(float(jc["rho"]), float(jc["E"]), float(jc["nu"]), float(jc["a"]),
                   float(jc["b"]), float(jc["n"]), c=float(jc["c"]), eps0=float(jc["eps0"]),
                   epsmax=float(jc["epsmax"]), sigmax=float(jc["sigmax"]))
        geo = solid_prop(qa=pr["qa"] or 1.1, qb=pr["qb"] or 0.05, qh=pr["h"] or 0.1)
        groups.append(HexaGroupSpec(ixs, mat, geo, jcvt=1 if int(pr["Iframe"]) == 2 else 0))
    icodt = np.zeros(numnod, np.int32)
    off = np.asarray(d["bcs_offsets"])
    bn = to_idx(np.asarray(d["bcs_nodes"]))
    for k, (tra, rot) in enumerate(zip(d["bcs_tra"], d["bcs_rot"])):
        icodt[bn[off[k]:off[k + 1]] - 1] |= _code_bits(str(tra), 1) | _code_bits(str(rot), 8)
    inr = np.zeros(numnod)
    rmats = []
    if rigid_cols:
        for nodes in rigid_material_bodies(np.concatenate(rigid_cols, axis=1)):
            xg, mass, axes, inertia = rigid_mat_init(X, ms, inr, nodes)
            rmats.append((nodes, xg, mass, axes, inertia))
    fx, fy = np.asarray(d["funct1"], np.float64).T
    xs, ys, t0, t1 = (float(v) for v in d["impvel_scale"])
    facx = 1.0 / (xs or 1.0)
    impvels = [(index[int(n)], int(d["impvel_dir"]), facx, ys or 1.0, t0, t1 or 1e30, fx, fy)
               for n in d["impvel_nodes"]]
    m = Model(name, X, np.zeros_like(X), ms, icodt, hexa=groups, IN=inr)
    m.rmats = rmats
    m.impvels = impvels
    dt = np.asarray(d["run_dt"])
    if dt[0] > 0:
        m.dtfac_solid = float(dt[0])
    return m

