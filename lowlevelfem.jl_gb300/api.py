"""Host-side mirror of LowLevelFEM.jl's assembly/solve API.

Function names, argument meanings and error behaviour follow the reference
(v1.13.31); every numerical operation runs in libllfem_gb300.so on the GPU.
This layer only moves arrays, resolves physical groups into node/element
sets, and wraps results in the reference's return types.

Reference entry points mirrored here:
  Material, elastic_constants            src/general.jl:99-203
  Problem                                src/general.jl:478-632
  stiffnessMatrix                        src/linear.jl:70-87, :190-330
  massMatrix                             src/linear.jl:1843-2004
  heatConductionMatrix                   src/heat.jl:28-137
  loadVector                             src/linear.jl:3088-3434
  constrainedDoFs / allDoFs / freeDoFs   src/general.jl:5289-5322, :5457-5492
  applyBoundaryConditions!               src/linear.jl:3505-3563
  solveDisplacement                      src/linear.jl:3711-3743, :3801-3870
  solveTemperature                       src/heat.jl:1020-1084
  solveField                             src/poisson.jl:1432-1546
  materialTangentMatrix                  src/nonlinear.jl:2083-2268
  initialStressMatrix                    src/nonlinear.jl:2417-2595
  internalForceVector                    src/nonlinear.jl:2738-2910
  ∇ / u∘∇ (grad)                         src/nabla.jl:77-311, src/operators.jl:2875-2881
  SystemMatrix + / - / *                 src/operators.jl:2411-2550
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .mesh import Mesh, current_mesh

SQRT_EPS = math.sqrt(np.finfo(float).eps)

_PTYPES = {
    "Solid": (_lib.SOLID, 3, 3, "u"),
    "PlaneStress": (_lib.PLANE_STRESS, 2, 2, "u"),
    "PlaneStrain": (_lib.PLANE_STRAIN, 2, 2, "u"),
    "HeatConduction": (_lib.HEAT_CONDUCTION, 3, 1, "T"),
    "PlaneHeatConduction": (_lib.PLANE_HEAT_CONDUCTION, 2, 1, "T"),
}


def _sym(s) -> str:
    s = str(s)
    return s[1:] if s.startswith(":") else s


# --------------------------------------------------------------------------
# Material
# --------------------------------------------------------------------------
def elastic_constants(E=None, nu=None, lam=None, mu=None, kappa=None):
    """E, ν, λ, μ, κ from any admissible pair (src/general.jl:142-203)."""
    given = {k for k, v in dict(E=E, nu=nu, lam=lam, mu=mu, kappa=kappa).items() if v is not None}
    n = len(given)
    if n == 0 or (n == 1 and "E" in given):
        E = 2.0e5 if n == 0 else E
        nu = 0.3
        mu = E / (2 * (1 + nu))
        lam = 2 * mu * nu / (1 - 2 * nu)
        kappa = E / (3 * (1 - 2 * nu))
    elif n == 1 and "kappa" in given:
        E = 2.0e5
        nu = (1 - E / (3 * kappa)) / 2
        mu = E / (2 * (1 + nu))
        lam = 2 * mu * nu / (1 - 2 * nu)
    elif n == 2 and given == {"E", "nu"}:
        mu = E / (2 * (1 + nu))
        lam = 2 * mu * nu / (1 - 2 * nu)
        kappa = E / (3 * (1 - 2 * nu))
    elif n == 2 and given == {"mu", "nu"}:
        E = 2 * mu * (1 + nu)
        lam = 2 * mu * nu / (1 - 2 * nu)
        kappa = E / (3 * (1 - 2 * nu))
    elif n == 2 and given == {"lam", "mu"}:
        nu = lam / (2 * (lam + mu))
        E = mu * (3 * lam + 2 * mu) / (lam + mu)
        kappa = lam + 2 * mu / 3
    elif n == 2 and given == {"kappa", "mu"}:
        lam = kappa - 2 * mu / 3
        nu = lam / (2 * (lam + mu))
        E = 2 * mu * (1 + nu)
    elif n < 2:
        raise ValueError("Insufficient elastic parameters. Specify at least E+ν, μ+ν, λ+μ, κ+μ, or E alone.")
    else:
        raise ValueError(f"Elastic constants are overdetermined: {sorted(given)}")
    return dict(E=E, nu=nu, lam=lam, mu=mu, kappa=kappa)


class Material:
    """Material(phName; type, E, ν, λ, μ, κ, ρ, k, c, α) (src/general.jl:99-140)."""

    def __init__(self, phName: str, type="Hooke", E=None, nu=None, lam=None, mu=None, kappa=None,
                 rho=7.85e-9, k=45.0, c=4.2e8, alpha=1.2e-5):
        t = _sym(type)
        if t not in ("Hooke", "StVenantKirchhoff", "NeoHookeCompressible", "JFO"):
            raise ValueError(f"Invalid material type: {t}")
        ec = elastic_constants(E=E, nu=nu, lam=lam, mu=mu, kappa=kappa)
        self.phName, self.type = phName, t
        self.E, self.nu, self.lam, self.mu, self.kappa = ec["E"], ec["nu"], ec["lam"], ec["mu"], ec["kappa"]
        self.rho, self.k, self.c, self.alpha = rho, k, c, alpha


material = Material


# --------------------------------------------------------------------------
# Problem
# --------------------------------------------------------------------------
class Problem:
    """Problem(materials; type, thickness, dim) on the current mesh
    (src/general.jl:478-632)."""

    def __init__(self, materials, type="Solid", thickness=1.0, dim=3, field=None, mesh: Mesh | None = None,
                 device: int | None = None):
        if not isinstance(materials, (list, tuple)):
            raise ValueError("Problem: materials are not arranged in a vector. Put them in [...]")
        t = _sym(type)
        if t == "VectorField":
            if dim not in (2, 3):
                raise ValueError("Problem: dimension of a :VectorField problem must be two or three.")
            self.type, self.dim, self.pdim, self.field = ("Solid" if dim == 3 else "PlaneStrain"), dim, dim, (field or "u")
            self.ptype = _lib.SOLID if dim == 3 else _lib.PLANE_STRAIN
        elif t == "ScalarField":
            self.type, self.dim, self.pdim, self.field = ("HeatConduction" if dim == 3 else "PlaneHeatConduction"), dim, 1, (field or "T")
            self.ptype = _lib.HEAT_CONDUCTION if dim == 3 else _lib.PLANE_HEAT_CONDUCTION
        elif t in _PTYPES:
            self.ptype, self.dim, self.pdim, self.field = _PTYPES[t]
            self.type = t
        else:
            raise ValueError(f"Problem type can be: `:Solid`, `:PlaneStress`, `:PlaneStrain`, "
                             f"`:PlaneHeatConduction`, `:HeatConduction`. Now problem type = {t} ????")
        self.material = list(materials)
        self.thickness = float(thickness)
        self.mesh = mesh if mesh is not None else current_mesh()
        if self.mesh.dim != self.dim:
            raise ValueError(f"Problem: dimension of the problem ({self.dim}) is different than the "
                             f"dimension of finite elements ({self.mesh.dim}).")
        self.non = self.mesh.non
        self.name = self.mesh.name
        self._device = device
        self._ctx_obj = None
        self._dmesh = None
        self._dpat = {}
        self._bmesh = {}

    @property
    def _ctx(self) -> _lib.Context:
        if self._ctx_obj is None:
            self._ctx_obj = _lib.default_context() if self._device is None else _lib.Context(self._device)
        return self._ctx_obj

    # element -> material index (elements outside every material group: -1)
    def element_materials(self) -> np.ndarray:
        em = np.full(self.mesh.nel, -1, dtype=np.int32)
        for i, m in enumerate(self.material):
            g = self.mesh.group(m.phName)
            if g.dim != self.dim:
                raise ValueError(f"Problem: material group '{m.phName}' has dimension {g.dim}, problem dimension {self.dim}.")
            em[_group_elements(self.mesh, g)] = i
        return em

    def device_mesh(self) -> _lib.DeviceMesh:
        if self._dmesh is None:
            dm = _lib.DeviceMesh(self._ctx, self.dim, self.mesh.xyz, self.mesh.conn, self.mesh.family, self.mesh.order)
            em = self.element_materials()
            dm.set_materials(None if np.all(em == 0) else em)
            self._dmesh = dm
        return self._dmesh

    def pattern(self, pdim: int | None = None) -> _lib.DevicePattern:
        p = self.pdim if pdim is None else pdim
        if p not in self._dpat:
            self._dpat[p] = _lib.DevicePattern(self.device_mesh(), p)
        return self._dpat[p]

    def boundary_mesh(self, name) -> _lib.DeviceMesh:
        """Device mesh of a boundary group, or of several groups of one element
        type (a tuple of names) as one element list in the given order."""
        key = name if isinstance(name, str) else tuple(name)
        if key not in self._bmesh:
            gs = [self.mesh.group(n) for n in ((key,) if isinstance(key, str) else key)]
            g = gs[0]
            if any(x.family != g.family or x.order != g.order for x in gs):
                raise ValueError("boundary_mesh: the groups hold different element types")
            conn = np.concatenate([x.conn for x in gs], axis=0)
            self._bmesh[key] = _lib.DeviceMesh(self._ctx, self.dim, self.mesh.xyz, conn, g.family, g.order)
        return self._bmesh[key]


Field = Problem


def _group_elements(mesh: Mesh, g) -> np.ndarray:
    if getattr(g, "elems", None) is not None:
        return g.elems
    if g.conn is not None and g.conn.shape == mesh.conn.shape and np.array_equal(g.conn, mesh.conn):
        return np.arange(mesh.nel)
    # match element rows of the group against the volume connectivity
    key = {tuple(r): i for i, r in enumerate(mesh.conn.tolist())}
    return np.array([key[tuple(r)] for r in g.conn.tolist()], dtype=np.int64)


# --------------------------------------------------------------------------
# Fields and system matrices
# --------------------------------------------------------------------------
@dataclass
class VectorField:
    a: np.ndarray                 # (ndof, nsteps)
    model: Problem
    type: str = "v3D"


@dataclass
class ScalarField:
    a: np.ndarray
    model: Problem
    type: str = "scalar"


@dataclass
class TensorField:
    """Tensor field, elementwise (A[e] holds 9*npe values, column-major 3x3
    per element node, the layout of src/nabla.jl:190-208) or nodal (a holds
    9 values per node, the same order)."""
    A: np.ndarray | None          # (nel, 9*npe), or None for a nodal field
    model: Problem
    type: str = "tensor"
    a: np.ndarray | None = None   # (9*non, 1) for a nodal field


def isElementwise(T) -> bool:
    """isElementwise (src/general.jl): the field holds element-node values."""
    return getattr(T, "A", None) is not None


def _field_for(problem: Problem, a: np.ndarray):
    a = a.reshape(-1, 1) if a.ndim == 1 else a
    if problem.pdim == 1:
        return ScalarField(a, problem)
    return VectorField(a, problem, "v3D" if problem.pdim == 3 else "v2D")


class SystemMatrix:
    """SystemMatrix(A::SparseMatrixCSC{Float64,Int64}, model) backed by a
    device matrix; the host CSC arrays are fetched on first use."""

    def __init__(self, dm: _lib.DeviceMatrix, model: Problem):
        self.dm = dm
        self.model = model
        self._csc = None

    def csc(self):
        """(colptr, rowval, nzval) as Julia's SparseMatrixCSC holds them (1-based)."""
        if self._csc is None:
            self._csc = self.dm.copy_csc()
        return self._csc

    @property
    def A(self):
        import scipy.sparse as sp
        c, r, v = self.csc()
        return sp.csc_matrix((v, r - 1, c - 1), shape=(self.dm.n, self.dm.n))

    @property
    def shape(self):
        return (self.dm.n, self.dm.n)

    def nnz(self) -> int:
        return self.dm.nnz()

    def __add__(self, o: "SystemMatrix"):
        return SystemMatrix(self.dm.axpby(1.0, 1.0, o.dm), self.model)

    def __sub__(self, o: "SystemMatrix"):
        return SystemMatrix(self.dm.axpby(1.0, -1.0, o.dm), self.model)

    def __rmul__(self, s: float):
        return SystemMatrix(self.dm.axpby(float(s), 0.0, self.dm), self.model)

    def __mul__(self, x):
        if np.isscalar(x):
            return self.__rmul__(x)
        if isinstance(x, (VectorField, ScalarField)):
            return _field_for(self.model, self.dm.spmv(x.a[:, 0]))
        return self.dm.spmv(np.asarray(x, dtype=np.float64))


# --------------------------------------------------------------------------
# Assembly
# --------------------------------------------------------------------------
def _form(precision) -> int:
    return _lib.FP32Q if str(precision).lower() in ("fp32", "fp32q", "mixed") else _lib.FP64


def stiffnessMatrix(problem: Problem, elements=(), forceOneThread=True, precision="fp64") -> SystemMatrix:
    """K = Σ BᵀDB b detJ w, CSC with dropzeros! (src/linear.jl:70-87, :190-330).
    `forceOneThread` is accepted for signature compatibility; the GPU path has
    no thread switch."""
    if problem.pdim != problem.dim or problem.type not in ("Solid", "PlaneStress", "PlaneStrain"):
        raise ValueError("constitutive_matrix: unsupported dim/type combo")
    ctx = problem._ctx
    E = np.array([m.E for m in problem.material])
    nu = np.array([m.nu for m in problem.material])
    h = _lib.C.c_void_p()
    dm, pat = problem.device_mesh(), problem.pattern()
    ctx.check(_lib.lib().llf_assemble_stiffness(ctx.h, dm.h, pat.h, problem.ptype, _lib.ptr(E, _lib.C.c_double),
                                                _lib.ptr(nu, _lib.C.c_double), len(E), problem.thickness,
                                                _form(precision), _lib.C.byref(h)), "stiffnessMatrix")
    return SystemMatrix(_lib.DeviceMatrix(ctx, h, pat), problem)


def autotune(problem: Problem, precision="fp64", trials=3) -> dict:
    """Tune the launch schedule of stiffnessMatrix(problem) on this problem's
    mesh and pattern (llf_autotune_stiffness): the chosen schedule is kept
    for every later assembly of this shape; results do not change.  Returns
    the tuner's report (candidates, times, the choice)."""
    import json
    ctx = problem._ctx
    E = np.array([m.E for m in problem.material])
    nu = np.array([m.nu for m in problem.material])
    dm, pat = problem.device_mesh(), problem.pattern()
    need = _lib.C.c_int64(0)
    buf = _lib.C.create_string_buffer(1 << 16)
    ctx.check(_lib.lib().llf_autotune_stiffness(ctx.h, dm.h, pat.h, problem.ptype, _lib.ptr(E, _lib.C.c_double),
                                                _lib.ptr(nu, _lib.C.c_double), len(E), problem.thickness,
                                                _form(precision), int(trials), buf, 1 << 16,
                                                _lib.C.byref(need)), "autotune")
    return json.loads(buf.value.decode())


def massMatrix(problem: Problem, lumped=True, precision="fp64") -> SystemMatrix:
    """M = ρ b Σ HᵀH detJ w, consistent or row-sum lumped (src/linear.jl:1843-2004)."""
    if problem.type not in ("Solid", "PlaneStress", "PlaneStrain"):
        raise ValueError(f"massMatrixSolid: unsupported dim={problem.dim}, type={problem.type}")
    ctx = problem._ctx
    rho = np.array([m.rho for m in problem.material])
    h = _lib.C.c_void_p()
    dm, pat = problem.device_mesh(), problem.pattern()
    ctx.check(_lib.lib().llf_assemble_mass(ctx.h, dm.h, pat.h, problem.ptype, _lib.ptr(rho, _lib.C.c_double),
                                           len(rho), problem.thickness, int(bool(lumped)), _form(precision),
                                           _lib.C.byref(h)), "massMatrix")
    return SystemMatrix(_lib.DeviceMatrix(ctx, h, pat), problem)


def heatCapacityMatrix(problem: Problem, elements=(), lumped=False, precision="fp64") -> SystemMatrix:
    """C = c ρ Σ HᵀH detJ w (b = 1 in 2D and 3D), consistent or row-sum lumped
    (src/heat.jl:257-376): the mass kernels on the scalar pattern with c ρ."""
    if problem.type not in ("HeatConduction", "PlaneHeatConduction"):
        raise ValueError(f"heatCapacityMatrix: dimension is {problem.dim}, problem type is {problem.type}.")
    ctx = problem._ctx
    crho = np.array([m.c * m.rho for m in problem.material])
    h = _lib.C.c_void_p()
    dm, pat = problem.device_mesh(), problem.pattern()
    ctx.check(_lib.lib().llf_assemble_mass(ctx.h, dm.h, pat.h, problem.ptype, _lib.ptr(crho, _lib.C.c_double),
                                           len(crho), problem.thickness, int(bool(lumped)), _form(precision),
                                           _lib.C.byref(h)), "heatCapacityMatrix")
    return SystemMatrix(_lib.DeviceMatrix(ctx, h, pat), problem)


def heatConductionMatrix(problem: Problem, elements=(), precision="fp64") -> SystemMatrix:
    """K_T = Σ ∇Nᵀ∇N k b detJ w (src/heat.jl:28-137)."""
    if problem.type not in ("HeatConduction", "PlaneHeatConduction"):
        raise ValueError(f"heatCondMatrixSolid: dimension is {problem.dim}, problem type is {problem.type}.")
    ctx = problem._ctx
    k = np.array([m.k for m in problem.material])
    h = _lib.C.c_void_p()
    dm, pat = problem.device_mesh(), problem.pattern()
    ctx.check(_lib.lib().llf_assemble_heat(ctx.h, dm.h, pat.h, problem.ptype, _lib.ptr(k, _lib.C.c_double),
                                           len(k), problem.thickness, _form(precision), _lib.C.byref(h)),
              "heatConductionMatrix")
    return SystemMatrix(_lib.DeviceMatrix(ctx, h, pat), problem)


# --------------------------------------------------------------------------
# Boundary conditions and loads
# --------------------------------------------------------------------------
class BoundaryCondition:
    """BoundaryCondition(phName; kwargs...) (src/general.jl:2480-2494)."""

    def __init__(self, phName: str, problem=None, **values):
        self.phName = phName
        self.problem = problem
        self.values = {k: v for k, v in values.items() if v is not None}


class LoadCondition(BoundaryCondition):
    """LoadCondition(phName; kwargs...) (src/general.jl:2589-2605)."""


def displacementConstraint(name, ux=None, uy=None, uz=None):
    return BoundaryCondition(name, ux=ux, uy=uy, uz=uz)


def temperatureConstraint(name, T=None):
    return BoundaryCondition(name, T=T)


def load(name, fx=None, fy=None, fz=None):
    return LoadCondition(name, fx=fx, fy=fy, fz=fz)


def heatFlux(name, qn=None):
    return LoadCondition(name, qn=qn)


def elasticSupport(name, kx=None, ky=None, kz=None):
    """elasticSupport(name; kx, ky, kz) (src/general.jl:4281-4285)."""
    if kx is None and ky is None and kz is None:
        raise ValueError("elasticSupport: at least one of kx, ky, kz, p must be specified.")
    return BoundaryCondition(name, kx=kx, ky=ky, kz=kz)


def heatConvection(name, h=None, Tinf=None):
    """heatConvection(name; h, T∞) (src/general.jl:4384-4388); the ambient
    temperature is stored under the reference's key "T∞"."""
    if h is None or Tinf is None:
        raise ValueError("heatSource: h and T∞ must be specified.")
    return BoundaryCondition(name, h=h, **{"T∞": Tinf})


def _component(problem: Problem, key: str):
    fld = problem.field
    if not key.startswith(fld):
        return None
    suffix = key[len(fld):]
    if problem.pdim == 1:
        return 0 if suffix in ("",) else None
    idx = {"x": 0, "y": 1, "z": 2}.get(suffix)
    if idx is None or idx >= problem.pdim:
        return None
    return idx


def constrainedDoFs(problem: Problem, supports) -> np.ndarray:
    """1-based constrained DoFs in the reference's order (unique of the
    per-condition, per-component, per-node list)."""
    dofs = []
    for bc in supports:
        if bc.problem is not None and bc.problem is not problem:
            continue
        nodes = problem.mesh.group(bc.phName).nodes
        for key in bc.values:
            c = _component(problem, key)
            if c is None:
                continue
            dofs.extend(((nodes - 1) * problem.pdim + c + 1).tolist())
    _, idx = np.unique(np.asarray(dofs, dtype=np.int64), return_index=True)
    return np.asarray(dofs, dtype=np.int64)[np.sort(idx)] if dofs else np.zeros(0, dtype=np.int64)


def allDoFs(problem: Problem) -> np.ndarray:
    nodes = []
    for m in problem.material:
        nodes.append(problem.mesh.group(m.phName).nodes)
    nodes = np.unique(np.concatenate(nodes))
    return np.concatenate([problem.pdim * nodes - (problem.pdim - p) for p in range(1, problem.pdim + 1)])


def freeDoFs(problem: Problem, supports) -> np.ndarray:
    c = set(constrainedDoFs(problem, supports).tolist())
    return np.array([d for d in allDoFs(problem).tolist() if d not in c], dtype=np.int64)


def _values_at(problem: Problem, nodes: np.ndarray, v):
    if callable(v):
        x = problem.mesh.xyz[nodes - 1]
        return np.array([float(v(*p)) for p in x])
    if isinstance(v, ScalarField):
        return v.a[nodes - 1, 0]
    return np.full(len(nodes), float(v))


def applyBoundaryConditions_(u, supports):
    """applyBoundaryConditions!(field, supports): write prescribed values
    (src/linear.jl:3505-3563)."""
    problem = u.model
    for bc in supports:
        if bc.problem is not None and bc.problem is not problem:
            continue
        nodes = problem.mesh.group(bc.phName).nodes
        for key, v in bc.values.items():
            c = _component(problem, key)
            if c is None:
                continue
            u.a[(nodes - 1) * problem.pdim + c, 0] = _values_at(problem, nodes, v)
    return u


def loadVector(problem: Problem, loads, F=None) -> VectorField | ScalarField:
    """Consistent nodal loads of LoadConditions on boundary groups
    (src/linear.jl:3088-3434).  Constant values are integrated exactly;
    function values are sampled at the group's nodes and interpolated with the
    shape functions.  With F (the deformation gradient, nodal or elementwise)
    the tractions on faces of a 3D body are follower loads F t
    (src/linear.jl:3333-3372)."""
    ndof = problem.pdim * problem.non
    f = np.zeros(ndof)
    ctx = problem._ctx
    Fn = None
    if F is not None:
        if problem.dim != 3 or problem.pdim != 3:
            raise ValueError("loadVector: follower loads need a 3D vector problem")
        Fn = _nodal_F(problem, F)
    for ld in loads:
        g = problem.mesh.group(ld.phName)
        keys = ["qn"] if problem.pdim == 1 else ["fx", "fy", "fz"][: problem.pdim]
        if problem.pdim == 1 and "qn" not in ld.values and "q" in ld.values:
            keys = ["q"]
        vals = [ld.values.get(k, 0.0) for k in keys]
        if g.dim == 0:
            if Fn is not None:
                raise NotImplementedError("loadVector: follower loads on point groups are not accelerated")
            for n in g.nodes:
                for c, v in enumerate(vals):
                    f[(n - 1) * problem.pdim + c] += float(v(*problem.mesh.xyz[n - 1]) if callable(v) else v)
            continue
        if g.dim != problem.dim - 1:
            raise ValueError(f"loadVector: dimension of the problem is {problem.dim}, dimension of load is {g.dim}.")
        bm = problem.boundary_mesh(ld.phName)
        const = all(np.isscalar(v) for v in vals)
        tconst = np.array([float(v) for v in vals]) if const else None
        tn = None
        if not const:
            tn = np.zeros(ndof)
            for c, v in enumerate(vals):
                tn[(g.nodes - 1) * problem.pdim + c] = _values_at(problem, g.nodes, v)
        if Fn is not None:
            ctx.check(_lib.lib().llf_load_vector_follower(ctx.h, bm.h, _lib.ptr(Fn, _lib.C.c_double),
                                                          _lib.ptr(tconst, _lib.C.c_double),
                                                          _lib.ptr(tn, _lib.C.c_double),
                                                          _lib.ptr(f, _lib.C.c_double), ndof), "loadVector")
            continue
        ctx.check(_lib.lib().llf_load_vector(ctx.h, bm.h, problem.dim, problem.pdim,
                                             _lib.ptr(tconst, _lib.C.c_double), _lib.ptr(tn, _lib.C.c_double),
                                             problem.thickness if problem.dim == 2 else 1.0,
                                             _lib.ptr(f, _lib.C.c_double), ndof), "loadVector")
    return _field_for(problem, f)


def elementsToNodes(T: TensorField) -> TensorField:
    """elementsToNodes (src/general.jl:5519-5640): the mean of the
    element-node values at every node, summed in element order."""
    if not isElementwise(T):
        return T
    problem = T.model
    A = _tensor_array(problem, T)
    out = np.zeros(9 * problem.non)
    ctx = problem._ctx
    ctx.check(_lib.lib().llf_elements_to_nodes(ctx.h, problem.device_mesh().h, 9, _lib.ptr(A, _lib.C.c_double),
                                               _lib.ptr(out, _lib.C.c_double)), "elementsToNodes")
    return TensorField(None, problem, a=out.reshape(-1, 1))


def _nodal_F(problem: Problem, F) -> np.ndarray:
    """F as 9 values per node (column-major 3x3), from a nodal or an
    elementwise TensorField or a (non, 9) array."""
    if isinstance(F, TensorField):
        F = elementsToNodes(F).a
    F = np.ascontiguousarray(np.asarray(F, dtype=np.float64).reshape(-1))
    if F.size != 9 * problem.non:
        raise ValueError(f"F must hold 9 values per node ({9 * problem.non}), got {F.size}")
    return F


def _boundary_runs(problem: Problem, conds, what):
    """Consecutive conditions whose groups share the element type, each
    group of dimension dim-1."""
    runs = []
    for bc in conds:
        g = problem.mesh.group(bc.phName)
        if g.dim != problem.dim - 1:
            raise NotImplementedError(f"{what}: only boundary groups of dimension {problem.dim - 1} are "
                                      f"accelerated (group {bc.phName!r} has dimension {g.dim})")
        if runs and (runs[-1][-1][1].family, runs[-1][-1][1].order) == (g.family, g.order):
            runs[-1].append((bc, g))
        else:
            runs.append([(bc, g)])
    return runs


def _element_values(problem: Problem, run, keys):
    """Per-element constants (nel, len(keys)) of a run, or, when one value is
    a function or a field, the values at every element's nodes
    (nel, npe, len(keys)).  Returns (constants, element-node values)."""
    vals = [[bc.values.get(k, 0.0) for k in keys] for bc, _ in run]
    nodal = any(not np.isscalar(v) for vs in vals for v in vs)
    parts = []
    for (bc, g), vs in zip(run, vals):
        if nodal:
            kn = np.zeros((problem.non, len(keys)))
            for c, v in enumerate(vs):
                kn[g.nodes - 1, c] = _values_at(problem, g.nodes, v)
            parts.append(kn[g.conn - 1])
        else:
            parts.append(np.tile(np.array([float(v) for v in vs]), (g.conn.shape[0], 1)))
    karr = np.ascontiguousarray(np.concatenate(parts, axis=0), dtype=np.float64)
    return (None, karr) if nodal else (karr, None)


def externalTangentFollower(problem: Problem, loads, F) -> SystemMatrix:
    """Tangent of follower traction loads fx, fy, fz on faces of a 3D body
    (src/nonlinear.jl:3053-3258), K_ext; the Newton matrix is
    K_mat + K_geo - K_ext.  F: the deformation gradient, nodal or
    elementwise (averaged to the nodes).  The loads' groups of one element
    type go in one call in load order."""
    if problem.dim != 3 or problem.pdim != 3:
        raise ValueError("externalTangentFollower: dim == 3 && pdim == 3 is required")
    loads = list(loads)
    for ld in loads:
        if "p" in ld.values:
            raise NotImplementedError("externalTangentFollower: pressure follower loads are not accelerated")
    Fn = _nodal_F(problem, F)
    ctx, pat = problem._ctx, problem.pattern()
    total = None
    for run in _boundary_runs(problem, loads, "externalTangentFollower"):
        te, ten = _element_values(problem, run, ["fx", "fy", "fz"])
        bm = problem.boundary_mesh(tuple(bc.phName for bc, _ in run))
        h = _lib.C.c_void_p()
        ctx.check(_lib.lib().llf_follower_tangent(ctx.h, pat.h, bm.h, _lib.ptr(Fn, _lib.C.c_double),
                                                  _lib.ptr(te, _lib.C.c_double), _lib.ptr(ten, _lib.C.c_double),
                                                  _lib.C.byref(h)), "externalTangentFollower")
        K = SystemMatrix(_lib.DeviceMatrix(ctx, h, pat), problem)
        total = K if total is None else total + K
    if total is None:
        raise ValueError("externalTangentFollower: no loads given")
    return total


def _support_matrix(problem: Problem, conds, keys, what) -> SystemMatrix:
    """Σ over the conditions' boundary groups of Hᵀ diag(k) H Ja w on the
    volume pattern.  Consecutive conditions on groups of one element type go
    to the device as one element list in condition order, which sums every
    entry in the order of the reference's single sparse() call; runs of
    different element types are added afterwards.  Constant values are used
    as they are; when a run holds a function value, every group of the run is
    sampled at its nodes and interpolated at the points."""
    ctx, pat = problem._ctx, problem.pattern()
    conds = list(conds)
    if not conds:
        raise ValueError(f"{what}: no conditions given")
    total = None
    for run in _boundary_runs(problem, conds, what):
        ke, ken = _element_values(problem, run, keys)
        bm = problem.boundary_mesh(tuple(bc.phName for bc, _ in run))
        h = _lib.C.c_void_p()
        ctx.check(_lib.lib().llf_assemble_support(ctx.h, pat.h, bm.h, _lib.ptr(ke, _lib.C.c_double),
                                                  _lib.ptr(ken, _lib.C.c_double),
                                                  problem.thickness if problem.dim == 2 else 1.0,
                                                  _lib.C.byref(h)), what)
        C = SystemMatrix(_lib.DeviceMatrix(ctx, h, pat), problem)
        total = C if total is None else total + C
    return total


def elasticSupportMatrix(problem: Problem, elSupports) -> SystemMatrix:
    """C = Σ Hᵀ diag(kx, ky, kz) H Ja w over the supports' boundary groups
    (src/linear.jl:2859-3005): elastic (Winkler) supports, added to K."""
    if not isinstance(elSupports, (list, tuple)):
        raise TypeError("elasticSupportMatrix: elastic supports are not arranged in a vector. Put them in [...]")
    return _support_matrix(problem, elSupports, ["kx", "ky", "kz"][: problem.pdim], "elasticSupportMatrix")


def heatConvectionMatrix(problem: Problem, heatConvection) -> SystemMatrix:
    """C = Σ Hᵀ h H Ja w over the convection groups (src/heat.jl:562-567)."""
    if not isinstance(heatConvection, (list, tuple)):
        raise TypeError("heatConvection: heat convections are not arranged in a vector. Put them in [...]")
    if problem.pdim != 1:
        raise ValueError("heatConvectionMatrix: the problem must be a heat conduction problem")
    return _support_matrix(problem, heatConvection, ["h"], "heatConvectionMatrix")


def heatConvectionVector(problem: Problem, heatConvection) -> ScalarField:
    """q = Σ Hᵀ (h T∞) Ja w over the convection groups (src/heat.jl:667-673,
    loadVector's h/T∞ branch src/linear.jl:3281-3285)."""
    if not isinstance(heatConvection, (list, tuple)):
        raise TypeError("heatConvectionVector: heat convections are not arranged in a vector. Put them in [...]")
    loads = []
    for bc in heatConvection:
        h, T = bc.values.get("h"), bc.values.get("T∞")
        if callable(h):
            raise ValueError("heatConvectionVector: h cannot be a function.")
        if h is None or T is None:
            raise ValueError("heatConvectionVector: h and T∞ must be specified.")
        qn = (lambda *x, T=T, h=h: float(T(*x)) * h) if callable(T) else float(T) * float(h)
        loads.append(LoadCondition(bc.phName, qn=qn))
    return loadVector(problem, loads)


def applyElasticSupport_(K: SystemMatrix, elSupports) -> SystemMatrix:
    """applyElasticSupport!(K, elSupports) (src/linear.jl:3648-3660): K += C.
    Returns the updated matrix (the device matrix is replaced in place)."""
    C = elasticSupportMatrix(K.model, list(elSupports))
    K.dm, K._csc = K.dm.axpby(1.0, 1.0, C.dm), None
    return K


def applyHeatConvection_(K: SystemMatrix, q, heatConvection):
    """applyHeatConvection!(K, q, heatConv) (src/heat.jl:969-981): K += C and
    q += the convection vector."""
    problem = K.model
    C = heatConvectionMatrix(problem, list(heatConvection))
    K.dm, K._csc = K.dm.axpby(1.0, 1.0, C.dm), None
    q.a += heatConvectionVector(problem, list(heatConvection)).a
    return None


# --------------------------------------------------------------------------
# Solves
# --------------------------------------------------------------------------
_PRECOND = {"identity": _lib.PRECOND_NONE, "none": _lib.PRECOND_NONE, None: _lib.PRECOND_NONE,
            "jacobi": _lib.PRECOND_JACOBI, "bjacobi": _lib.PRECOND_BJACOBI,
            "blockjacobi": _lib.PRECOND_BJACOBI, "ic0": _lib.PRECOND_IC0, "ichol": _lib.PRECOND_IC0}

# tolerance used when the caller asks for the reference's direct solve
DIRECT_RELTOL = 1e-13


def _solve(K: SystemMatrix, f, supports, iterative, reltol, maxiter, preconditioner):
    problem = K.model
    u = _field_for(problem, np.zeros(problem.pdim * problem.non))
    applyBoundaryConditions_(u, supports)
    fixed = np.zeros(problem.pdim * problem.non, dtype=np.uint8)
    cd = constrainedDoFs(problem, supports)
    fixed[cd - 1] = 1
    fa = f.a[:, 0] if hasattr(f, "a") else np.asarray(f, dtype=np.float64)
    if iterative:
        prec = _PRECOND[preconditioner.lower() if isinstance(preconditioner, str) else preconditioner]
        tol = reltol
    else:
        prec, tol = _lib.PRECOND_BJACOBI, DIRECT_RELTOL
        maxiter = max(maxiter, 20 * problem.pdim * problem.non)
    x, it, rr = K.dm.pcg(fa, u.a[:, 0], fixed, precond=prec, reltol=tol, maxiter=maxiter,
                         raise_on_fail=not iterative)
    u.a[:, 0] = x
    u.iterations, u.relres = it, rr
    return u


def solveDisplacement(problem_or_K, f=None, load=(), support=(), elasticSupport=(), condensed=True,
                      iterative=False, reltol=SQRT_EPS, maxiter=None, preconditioner="identity", ordering=True):
    """solveDisplacement(problem; load, support, ...) or solveDisplacement(K, f; support, ...)
    (src/linear.jl:3711-3743, :3801-3870).  Both the condensed and the
    non-condensed variants solve K[free,free] u_f = f_f - K[free,fixed] u_c.
    With iterative=false (the reference's direct `\\`) the GPU runs
    block-Jacobi PCG to a relative residual of 1e-13."""
    if isinstance(problem_or_K, SystemMatrix):
        K = problem_or_K
        if f is None:
            raise ValueError("solveDisplacement(K, f): f is required")
    else:
        problem = problem_or_K
        K = stiffnessMatrix(problem)
        if elasticSupport:
            applyElasticSupport_(K, elasticSupport)
        f = loadVector(problem, list(load))
    pr = K.model
    maxiter = pr.non * pr.dim if maxiter is None else maxiter
    return _solve(K, f, list(support), iterative, reltol, maxiter, preconditioner)


def solveTemperature(problem_or_K, q=None, heatFlux=(), temperatureConstraint=(), heatConvection=(),
                     iterative=False, reltol=SQRT_EPS, maxiter=None, preconditioner="identity"):
    """solveTemperature(problem; heatFlux, temperatureConstraint, heatConvection) or
    solveTemperature(K, q; temperatureConstraint) (src/heat.jl:1020-1084)."""
    if isinstance(problem_or_K, SystemMatrix):
        K = problem_or_K
    else:
        problem = problem_or_K
        K = heatConductionMatrix(problem)
        q = loadVector(problem, list(heatFlux))
        if heatConvection:
            applyHeatConvection_(K, q, heatConvection)
    pr = K.model
    maxiter = pr.non * pr.dim if maxiter is None else maxiter
    return _solve(K, q, list(temperatureConstraint), iterative, reltol, maxiter, preconditioner)


def FDM(K: SystemMatrix, C: SystemMatrix, q, bc, TT0, n: int, dt: float, theta: float = 0.5,
        preconditioner="bjacobi", reltol=DIRECT_RELTOL, maxiter=None):
    """Transient heat conduction by the theta-method, FDM(K, C, q, bc, TT0,
    n, Δt; ϑ) (src/heat.jl:1466-1616): n states T(0), T(Δt), ... with
    (C + ϑΔtK) T^{n+1} = (C − (1−ϑ)ΔtK) T^n + Δt q^{n+ϑ} on the free DoFs, or
    the explicit update for ϑ = 0 with a lumped C.  The whole time loop runs
    on the device: the reference's LU back-substitutions become PCG solves to
    `reltol` with the preconditioner built once.  Returns a field whose `a`
    holds the n states as columns and `t` the times."""
    problem = K.model
    if C.model is not problem or q.model is not problem or TT0.model is not problem:
        raise ValueError("FDM: K, C, q and TT0 must belong to the same model.")
    if n < 2:
        raise ValueError("FDM: n must be at least 2.")
    if not dt > 0:
        raise ValueError("FDM: Δt must be positive.")
    if not 0.0 <= theta <= 1.0:
        raise ValueError("FDM: ϑ must be between 0 and 1.")
    ndof = problem.pdim * problem.non
    qa = np.asarray(q.a, dtype=np.float64).reshape(ndof, -1)
    if qa.shape[1] not in (1, n):
        raise ValueError("FDM: number of time steps in q must be 1 or n.")
    T = np.zeros((n, ndof))                       # row i = the state at step i
    T[0] = np.asarray(TT0.a, dtype=np.float64).reshape(ndof, -1)[:, 0]
    u = _field_for(problem, np.zeros(ndof))
    applyBoundaryConditions_(u, list(bc))
    fixed = np.zeros(ndof, dtype=np.uint8)
    cd = constrainedDoFs(problem, list(bc))
    fixed[cd - 1] = 1
    T[:, cd - 1] = u.a[cd - 1, 0]                # prescribed in every step, the initial one included
    qt = np.ascontiguousarray(qa.T)
    prec = _PRECOND[preconditioner.lower() if isinstance(preconditioner, str) else preconditioner]
    maxiter = 20 * ndof if maxiter is None else maxiter
    it = _lib.C.c_int64(0)
    ctx = problem._ctx
    ctx.check(_lib.lib().llf_heat_fdm(ctx.h, K.dm.h, C.dm.h, _lib.ptr(qt, _lib.C.c_double), qt.shape[0],
                                      _lib.ptr(T, _lib.C.c_double), _lib.ptr(fixed, _lib.C.c_uint8), n, float(dt),
                                      float(theta), prec, float(reltol), int(maxiter), _lib.C.byref(it)), "FDM")
    out = _field_for(problem, np.ascontiguousarray(T.T))
    out.t = np.arange(n) * float(dt)
    out.iterations = it.value
    return out


def solveField(K: SystemMatrix, f, support=(), iterative=False, reltol=SQRT_EPS, maxiter=None,
               preconditioner="identity", ordering=True):
    """solveField(K, f; support, iterative, reltol, maxiter, preconditioner)
    (src/poisson.jl:1432-1546)."""
    pr = K.model
    maxiter = pr.non * pr.dim if maxiter is None else maxiter
    return _solve(K, f, list(support), iterative, reltol, maxiter, preconditioner)


def solveFieldBatched(K: SystemMatrix, f, support=(), node_offsets=None, iterative=True, reltol=SQRT_EPS,
                      maxiter=None, preconditioner="jacobi", precision="fp64"):
    """Many independent systems at once: K is the block-diagonal matrix of a
    batch (concat_meshes), instance i owning nodes node_offsets[i]..[i+1]-1
    (node_offsets=None: one system).  Every instance runs its own CG (own
    scalars and stopping rule) inside the same launches; instance i's result
    is bit-identical to solving it alone.  precision="mixed" runs the
    iterations in FP32 with FP64 reliable updates (llf_pcg_mixed): the
    stopping test is still on the FP64 residual.  Returns the field and
    per-instance iteration counts / residuals."""
    problem = K.model
    if node_offsets is None:
        node_offsets = [0, problem.non]
    if precision not in ("fp64", "mixed"):
        raise ValueError(f"solveFieldBatched: precision {precision!r} (fp64 or mixed)")
    u = _field_for(problem, np.zeros(problem.pdim * problem.non))
    applyBoundaryConditions_(u, list(support))
    fixed = np.zeros(problem.pdim * problem.non, dtype=np.uint8)
    cd = constrainedDoFs(problem, list(support))
    fixed[cd - 1] = 1
    fa = f.a[:, 0] if hasattr(f, "a") else np.asarray(f, dtype=np.float64)
    prec = _PRECOND[preconditioner.lower() if isinstance(preconditioner, str) else preconditioner]
    if not iterative:
        prec, reltol = _lib.PRECOND_BJACOBI, DIRECT_RELTOL
    seg = np.asarray(node_offsets, dtype=np.int64) * problem.pdim
    maxiter = problem.non * problem.dim if maxiter is None else maxiter
    x, its, rr = K.dm.pcg_batched(fa, u.a[:, 0], fixed, seg, precond=prec, reltol=reltol, maxiter=maxiter,
                                  raise_on_fail=not iterative, mixed=precision == "mixed")
    u.a[:, 0] = x
    u.iterations, u.relres = its, rr
    return u


# --------------------------------------------------------------------------
# Total Lagrangian
# --------------------------------------------------------------------------
_LAWS = {"NeoHookeCompressible": _lib.LAW_NEOHOOKE_COMP, "StVenantKirchhoff": _lib.LAW_SVK,
         "neo-hooke": _lib.LAW_NEOHOOKE_COMP, "svk": _lib.LAW_SVK}


def _law(energy, params, C=None):
    if C is not None:
        Cm = np.asarray(C, dtype=np.float64)
        if Cm.shape != (6, 6):
            raise ValueError("C must be a 6x6 Voigt matrix")
        return _lib.LAW_CONSTANT_C, np.ascontiguousarray(Cm.T).ravel()
    if energy is None:
        raise ValueError("give either C or energy")
    law = _LAWS.get(energy if isinstance(energy, str) else getattr(energy, "law", None))
    if law is None:
        raise ValueError(f"energy {energy!r}: built-in laws are {sorted(_LAWS)}")
    p = params or {}
    mu = float(p.get("mu", p.get("μ", 1.0)))
    lam = float(p.get("lambda", p.get("λ", 10.0)))
    return law, np.array([mu, lam])


def _tensor_array(problem: Problem, T) -> np.ndarray:
    """Elementwise (nel, 9*npe) values of a tensor field; a nodal field is
    taken at every element's nodes (nodesToElements, src/general.jl:5671)."""
    if isinstance(T, TensorField) and T.A is None:
        m = problem.mesh
        return np.ascontiguousarray(np.asarray(T.a, dtype=np.float64).reshape(-1, 9)[m.conn - 1]
                                    .reshape(m.nel, 9 * m.npe))
    A = T.A if isinstance(T, TensorField) else np.asarray(T)
    A = np.ascontiguousarray(A, dtype=np.float64)
    if A.shape != (problem.mesh.nel, 9 * problem.mesh.npe):
        raise ValueError(f"elementwise tensor field must be (nel, 9*npe) = ({problem.mesh.nel}, {9 * problem.mesh.npe})")
    return A


def grad(u, add_identity=False) -> TensorField:
    """u ∘ ∇: elementwise nodal gradient T[i,j] = ∂u_i/∂X_j (src/nabla.jl:77-311)."""
    problem = u.model
    ua = np.ascontiguousarray(u.a[:, 0], dtype=np.float64)
    out = np.zeros((problem.mesh.nel, 9 * problem.mesh.npe))
    ctx = problem._ctx
    ctx.check(_lib.lib().llf_grad_elementwise(ctx.h, problem.device_mesh().h, _lib.ptr(ua, _lib.C.c_double),
                                              int(add_identity), _lib.ptr(out, _lib.C.c_double)), "grad")
    return TensorField(out, problem)


def deformationGradient(u) -> TensorField:
    """F = I + u ∘ ∇."""
    return grad(u, add_identity=True)


def materialTangentMatrix(problem: Problem, F, C=None, energy=None, params=None) -> SystemMatrix:
    """K_mat = Σ B(F)ᵀ ℂ B(F) detJ0 w (src/nonlinear.jl:2083-2268)."""
    if (C is None) == (energy is None):
        raise AssertionError("xor(C !== nothing, energy !== nothing)")
    law, prm = _law(energy, params, C)
    Fa = _tensor_array(problem, F)
    ctx = problem._ctx
    h = _lib.C.c_void_p()
    dm, pat = problem.device_mesh(), problem.pattern()
    ctx.check(_lib.lib().llf_tl_material_tangent(ctx.h, dm.h, pat.h, _lib.ptr(Fa, _lib.C.c_double), law,
                                                 _lib.ptr(prm, _lib.C.c_double), len(prm), _lib.C.byref(h)),
              "materialTangentMatrix")
    return SystemMatrix(_lib.DeviceMatrix(ctx, h, pat), problem)


def tangentMatrix(problem: Problem, F, energy="NeoHookeCompressible", params=None, precision="fp64") -> SystemMatrix:
    """Consistent Newton tangent K_mat + K_geo from F in one pass (the exact
    derivative of internalForceVector for the same F); the reference's Newton
    loops sum materialTangentMatrix(F) and initialStressMatrix(C).
    precision="tf32x3": the element contraction on the tensor cores (split
    TF32 products, FP32 accumulation; for high-order elements)."""
    law, prm = _law(energy, params)
    Fa = _tensor_array(problem, F)
    ctx = problem._ctx
    h = _lib.C.c_void_p()
    dm, pat = problem.device_mesh(), problem.pattern()
    form = {"fp64": 0, "tf32x3": 2}[precision]
    ctx.check(_lib.lib().llf_tl_tangent_form(ctx.h, dm.h, pat.h, _lib.ptr(Fa, _lib.C.c_double), law,
                                             _lib.ptr(prm, _lib.C.c_double), len(prm), form, _lib.C.byref(h)),
              "tangentMatrix")
    return SystemMatrix(_lib.DeviceMatrix(ctx, h, pat), problem)


def solveDeformation(problem: Problem, support=(), load=(), energy="NeoHookeCompressible", params=None,
                     steps=10, tol=1e-8, maxit=25, reltol=1e-10, preconditioner="bjacobi", callback=None,
                     tangent="fp64"):
    """Total Lagrangian Newton solution in `steps` proportional load steps:
    prescribed displacements and external loads are ramped linearly; every
    Newton iteration evaluates F = I + u∘∇, f_int and the consistent tangent on
    the GPU and solves K du = f_ext - f_int for du with the increments of the
    prescribed values on the constrained DoFs.  Converged when the FP64
    residual on the free DoFs drops below tol times its value at the start of
    the step (or below tol times |f_ext| when that is larger).  Returns u and
    per-iteration records (step, iteration, residual norm, CG iterations).
    tangent="tf32x3" assembles the tangent on the tensor cores (split TF32
    products): the residual and the update stay FP64, so the iteration still
    converges to the FP64 tolerance, a little less than quadratically."""
    n = problem.pdim * problem.non
    u = _field_for(problem, np.zeros(n))
    target = _field_for(problem, np.zeros(n))
    applyBoundaryConditions_(target, list(support))
    fixed = np.zeros(n, dtype=np.uint8)
    fixed[constrainedDoFs(problem, list(support)) - 1] = 1
    fext_full = loadVector(problem, list(load)).a[:, 0] if load else np.zeros(n)
    free = fixed == 0
    history = []
    prec = _PRECOND[preconditioner]
    for step in range(1, steps + 1):
        lam = step / steps
        fext = lam * fext_full
        res0 = None
        for it in range(maxit):
            F = grad(u, add_identity=True)
            fint = internalForceVector(problem, F=F, energy=energy, params=params).a[:, 0]
            r = fext - fint
            r[~free] = 0.0
            rn = float(np.linalg.norm(r))
            du_fixed = np.where(free, 0.0, lam * target.a[:, 0] - u.a[:, 0])
            history.append({"step": step, "iter": it, "residual": rn})
            if not np.any(du_fixed != 0.0):
                if res0 is None:   # first equilibrium residual of the step
                    res0 = max(rn, float(np.linalg.norm(fext)), 1e-300)
                if rn <= tol * res0:
                    break
            K = tangentMatrix(problem, F, energy=energy, params=params, precision=tangent)
            x, cg_it, _ = K.dm.pcg(r, du_fixed, fixed, precond=prec, reltol=reltol, maxiter=20 * n,
                                   raise_on_fail=True)
            history[-1]["cg_iterations"] = cg_it
            u.a[:, 0] += x
            if callback:
                callback(step, it, rn)
    u.history = history
    return u


def initialStressMatrix(problem: Problem, S=None, energy=None, params=None, C=None) -> SystemMatrix:
    """K_geo[ai,bi] = Σ ∇Naᵀ S ∇Nb detJ0 w (src/nonlinear.jl:2417-2595);
    S given, or computed from the Cauchy-Green field C with `energy`."""
    if (S is None) == (energy is None):
        raise AssertionError("xor(stress !== nothing, energy !== nothing)")
    ctx = problem._ctx
    h = _lib.C.c_void_p()
    dm, pat = problem.device_mesh(), problem.pattern()
    if S is not None:
        Sa = _tensor_array(problem, S)
        ctx.check(_lib.lib().llf_tl_initial_stress(ctx.h, dm.h, pat.h, _lib.ptr(Sa, _lib.C.c_double), None,
                                                   0, None, 0, _lib.C.byref(h)), "initialStressMatrix")
    else:
        law, prm = _law(energy, params)
        Ca = _tensor_array(problem, C)
        ctx.check(_lib.lib().llf_tl_initial_stress(ctx.h, dm.h, pat.h, None, _lib.ptr(Ca, _lib.C.c_double),
                                                   law, _lib.ptr(prm, _lib.C.c_double), len(prm),
                                                   _lib.C.byref(h)), "initialStressMatrix")
    return SystemMatrix(_lib.DeviceMatrix(ctx, h, pat), problem)


def internalForceVector(problem: Problem, P=None, F=None, energy=None, params=None) -> VectorField:
    """f_int[ai] = Σ P_iJ ∂Na/∂X_J detJ0 w (src/nonlinear.jl:2738-2910)."""
    if (P is None) == (energy is None):
        raise AssertionError("Either provide `P` (TensorField), or provide (`energy`, `params`, `F`)")
    ctx = problem._ctx
    f = np.zeros(3 * problem.non)
    dm = problem.device_mesh()
    if P is not None:
        Pa = _tensor_array(problem, P)
        ctx.check(_lib.lib().llf_tl_internal_force(ctx.h, dm.h, _lib.ptr(Pa, _lib.C.c_double), None, 0, None, 0,
                                                   _lib.ptr(f, _lib.C.c_double)), "internalForceVector")
    else:
        if F is None:
            raise AssertionError("F is required with energy")
        law, prm = _law(energy, params)
        Fa = _tensor_array(problem, F)
        ctx.check(_lib.lib().llf_tl_internal_force(ctx.h, dm.h, None, _lib.ptr(Fa, _lib.C.c_double), law,
                                                   _lib.ptr(prm, _lib.C.c_double), len(prm),
                                                   _lib.ptr(f, _lib.C.c_double)), "internalForceVector")
    return VectorField(f.reshape(-1, 1), problem, "v3D")
