"""Spin systems and their interaction terms, API-compatible with
``muspinsim/spinsys.py``.

Host-side construction of the field-independent Hamiltonian from Zeeman,
hyperfine, dipolar and quadrupolar terms (small sparse matrices built once
per system).  The per-orientation work -- adding the rotated Zeeman field,
diagonalising, evolving -- happens on the GPU (``hamiltonian.py``,
``experiment.py``).
"""

import logging
from numbers import Number

import numpy as np
import scipy.constants as cnst
from scipy import sparse

from muspinsim_gb300.constants import EFG_2_MHZ, gyromagnetic_ratio, quadrupole_moment, spin
from muspinsim_gb300.hamiltonian import Hamiltonian
from muspinsim_gb300.spinop import Clonable, SpinOperator


# Kronecker-embedded operators keyed by (quantum numbers, include_only_given,
# axes per spin): many systems of a batch share their spins' structure.
_EMBED_CACHE = {}
_EMBED_CACHE_MAX = 65536


class InteractionTerm(Clonable):
    """T_{ab...} S^a_i S^b_j ... (muspinsim/spinsys.py:22-92)."""

    def __init__(self, spinsys, indices=[], tensor=0, label=None):
        self._spinsys = spinsys
        self._indices = np.array(indices)
        self._tensor = np.array(tensor)
        self._label = "Term" if label is None else label
        if np.any(np.array(self._tensor.shape) != 3):
            raise ValueError("Tensor is not fully three-dimensional")
        self._recalc_operator()

    def _recalc_operator(self):
        """Sum over all tensor index tuples of the Kronecker-embedded spin
        operators; a same-spin pair (quadrupole) multiplies S^a_i S^b_i
        (muspinsim/spinsys.py:34-69).  With Celio's method the operator
        spans only the term's own spins (in ascending spin order)."""
        total = None
        d = len(self._tensor.shape)
        tuples = np.indices(self._tensor.shape).reshape((d, -1)).T if d > 0 else [[]]
        only = bool(self._spinsys.celio_k)
        for ii in tuples:
            if len(self._indices) == 2 and self._indices[0] == self._indices[1]:
                spec = {int(self._indices[0]): ["xyz"[ii[0]], "xyz"[ii[1]]]}
            else:
                spec = {int(ind): "xyz"[ii[k]] for k, ind in enumerate(self._indices)}
            op = self._spinsys.operator(spec, include_only_given=only) * self._tensor[tuple(ii)]
            total = op if total is None else total + op
        self._operator = total

    @property
    def label(self):
        return self._label

    @property
    def indices(self):
        return tuple(self._indices)

    @property
    def tensor(self):
        return np.array(self._tensor)

    @property
    def operator(self):
        return self._operator.clone()

    @property
    def matrix(self):
        return self._operator.matrix

    def __repr__(self):
        return self.label


class SingleTerm(InteractionTerm):
    def __init__(self, spinsys, i, vector, label="Single"):
        super(SingleTerm, self).__init__(spinsys, [i], vector, label)

    @property
    def i(self):
        return self._indices[0]

    def rotate(self, rotmat):
        """v R^T (muspinsim/spinsys.py:103-110)."""
        R = np.array(rotmat)
        return SingleTerm(self._spinsys, self.i, np.dot(self._tensor, R.T), self._label)

    def __repr__(self):
        return "{0} {{ S_{1} * {2} }}".format(self._label, self.i, self._tensor)


class DoubleTerm(InteractionTerm):
    def __init__(self, spinsys, i, j, matrix, label="Double"):
        super(DoubleTerm, self).__init__(spinsys, [i, j], matrix, label)

    @property
    def i(self):
        return self._indices[0]

    @property
    def j(self):
        return self._indices[1]

    def rotate(self, rotmat):
        """R M R^T (muspinsim/spinsys.py:128-135)."""
        R = np.array(rotmat)
        M = np.linalg.multi_dot([R, self._tensor, R.T])
        return DoubleTerm(self._spinsys, self.i, self.j, M, self._label)

    def __repr__(self):
        return "{0} {{ S_{1} * [{2} {3} {4}] * S_{5} }}".format(
            self._label, self.i, *self._tensor, self.j
        )


class DissipationTerm(Clonable):
    """Container of a dissipation operator and rate (muspinsim/spinsys.py:
    143-158)."""

    def __init__(self, operator, gamma=0.0):
        self._op = operator
        self._g = gamma

    @property
    def operator(self):
        return self._op

    @property
    def gamma(self):
        return self._g

    @property
    def tuple(self):
        return (self._op, self._g)


class SpinSystem(Clonable):
    """Particles with spin and their interaction terms
    (muspinsim/spinsys.py:161-637)."""

    def __init__(self, spins=None, celio_k=0):
        if spins is None:
            spins = []
        gammas, Qs, Is, operators = [], [], [], []
        for s in spins:
            el, iso = s if isinstance(s, tuple) else (s, None)
            gammas.append(gyromagnetic_ratio(el, iso))
            Qs.append(quadrupole_moment(el, iso))
            Is.append(spin(el, iso))
            operators.append({a: SpinOperator.from_axes(Is[-1], a) for a in "xyz+-0"})
        self._spins = list(spins)
        self._gammas = np.array(gammas)
        self._Qs = np.array(Qs)
        self._Is = np.array(Is)
        self._dim = tuple((2 * self._Is + 1).astype(int))
        self._operators = operators
        self._terms = []
        self._dissip_terms = []
        self._celio_k = celio_k
        snames = ["{1}{0}".format(*s) if isinstance(s, tuple) else str(s) for s in self._spins]
        logging.info("Created spin system with spins:")
        logging.info("\t\t%s", " ".join(snames))

    @property
    def spins(self):
        return list(self._spins)

    @property
    def celio_k(self):
        return self._celio_k

    @property
    def gammas(self):
        return self._gammas.copy()

    @property
    def Qs(self):
        return self._Qs.copy()

    @property
    def Is(self):
        return self._Is.copy()

    @property
    def dimension(self):
        return self._dim

    @property
    def terms(self):
        return list(self._terms)

    @property
    def is_dissipative(self):
        return (np.array([t.gamma for t in self._dissip_terms]) != 0.0).any()

    def _check_index(self, i, name="i"):
        if i < 0 or i >= len(self._spins):
            raise ValueError(f"Invalid index {name}")

    def add_term(self, indices, tensor, label="Term"):
        for i in indices:
            self._check_index(i)
        term = InteractionTerm(self, indices, np.array(tensor), label=label)
        self._terms.append(term)
        return term

    def add_linear_term(self, i, vector, label="Single"):
        self._check_index(i)
        term = SingleTerm(self, i, np.array(vector), label=label)
        self._terms.append(term)
        return term

    def add_bilinear_term(self, i, j, matrix, label="Double"):
        self._check_index(i, "i")
        self._check_index(j, "j")
        term = DoubleTerm(self, i, j, np.array(matrix), label=label)
        self._terms.append(term)
        return term

    def add_zeeman_term(self, i, B):
        """gamma_i B . S_i, scalar B along z (muspinsim/spinsys.py:354-375)."""
        if isinstance(B, Number):
            B = [0, 0, B]
        B = np.array(B)
        logging.info("Adding Zeeman term to spin %s", i + 1)
        return self.add_linear_term(i, B * self.gamma(i), "Zeeman")

    def add_dipolar_term(self, i, j, r):
        """Point-dipole coupling from the vector r (Angstrom) between spins i
        and j, in MHz (muspinsim/spinsys.py:377-413)."""
        if i == j:
            raise ValueError("Can not set up dipolar coupling with itself")
        r = np.array(r)
        g_i = self.gamma(i)
        g_j = self.gamma(j)
        rnorm = np.linalg.norm(r)
        D = -(np.eye(3) - 3.0 / rnorm**2.0 * r[:, None] * r[None, :])
        dij = -(cnst.mu_0 * cnst.hbar * (g_i * g_j * 1e6)) / (2 * (rnorm * 1e-10) ** 3)
        D *= dij
        logging.info("Adding dipolar term to spins %s-%s", i + 1, j + 1)
        return self.add_bilinear_term(i, j, D, "Dipolar")

    def add_quadrupolar_term(self, i, EFG):
        """EFG_2_MHZ Q / (2I(2I-1)) EFG on spin i, I >= 1
        (muspinsim/spinsys.py:415-442)."""
        EFG = np.array(EFG)
        Q = self.Q(i)
        I = self.I(i)
        if I == 0.5:
            raise ValueError("Can not set up quadrupolar coupling for spin 1/2 particle")
        Qtens = EFG_2_MHZ * Q / (2 * I * (2 * I - 1)) * EFG
        logging.info("Adding quadrupolar term to spin %s", i + 1)
        return self.add_bilinear_term(i, i, Qtens, "Quadrupolar")

    def remove_term(self, term):
        self._terms.remove(term)

    def clear_terms(self):
        for t in list(self._terms):
            self.remove_term(t)

    def add_dissipative_term(self, op, d=0.0):
        term = DissipationTerm(op, d)
        self._dissip_terms.append(term)
        return term

    def remove_dissipative_term(self, term):
        self._dissip_terms.remove(term)

    def clear_dissipative_terms(self):
        for t in list(self._dissip_terms):
            self.remove_dissipative_term(t)

    def gamma(self, i):
        return self._gammas[i]

    def Q(self, i):
        return self._Qs[i]

    def I(self, i):  # noqa: E743
        return self._Is[i]

    def operator(self, terms=None, include_only_given=False):
        """Kronecker embedding of single-spin operators, spin 0 slowest
        (muspinsim/spinsys.py:545-592).  A list of axes for one index is
        multiplied in order.  The embedding depends only on the spins'
        quantum numbers and the requested axes, so it is cached across
        terms and systems (a copy is returned)."""
        if terms is None:
            terms = {}
        key = (tuple(float(x) for x in self._Is), bool(include_only_given),
               tuple(sorted((int(i), tuple(v) if isinstance(v, list) else v)
                            for i, v in terms.items())))
        hit = _EMBED_CACHE.get(key)
        if hit is not None:
            return hit.clone()
        M = self._embed(terms, include_only_given)
        if len(_EMBED_CACHE) < _EMBED_CACHE_MAX:
            _EMBED_CACHE[key] = M.clone()
        return M

    def _embed(self, terms, include_only_given):
        ops = []
        for i in range(len(self)):
            spec = terms.get(i, None if include_only_given else "0")
            if not spec:
                continue
            if isinstance(spec, list):
                o = self._operators[i][spec[0]]
                for a in spec[1:]:
                    o = o * self._operators[i][a]
            else:
                o = self._operators[i][spec]
            ops.append(o)
        M = ops[0]
        for o in ops[1:]:
            M = M.kron(o)
        return M

    def rotate(self, rotmat=np.eye(3)):
        """Copy with every term rotated (muspinsim/spinsys.py:594-611)."""
        terms = self._terms
        self._terms = []
        rssys = self.clone()
        self._terms = terms
        try:
            rssys._terms = [t.rotate(rotmat) for t in terms]
        except AttributeError as exc:
            raise RuntimeError("Can only rotate SpinSystems containing Single or Double terms") from exc
        for t in rssys._terms:
            t._spinsys = rssys
        return rssys

    def _cached(self, name, build):
        """Dense matrices derived from the term list, rebuilt only when the
        list of terms changes (terms are immutable once created)."""
        key = (name, tuple(id(t) for t in self._terms))
        cache = self.__dict__.setdefault("_matrix_cache", {})
        if key not in cache:
            cache.clear() if len(cache) > 8 else None
            cache[key] = build()
        return cache[key]

    def hamiltonian_matrix(self):
        """Dense sum of the term matrices (cached per term list)."""

        def build():
            n = int(np.prod(self.dimension))
            H = np.zeros((n, n), dtype=complex)
            for t in self._terms:
                H += t.matrix.toarray() if sparse.issparse(t.matrix) else t.matrix
            return H

        return self._cached("H", build).copy()

    @property
    def hamiltonian(self):
        """Hsys = sum of term matrices (muspinsim/spinsys.py:613-626), or a
        CelioHamiltonian of the terms with Celio's method."""
        if self._celio_k:
            from muspinsim_gb300.celio import CelioHamiltonian

            return CelioHamiltonian(self._terms, self._celio_k, self)
        if len(self._terms) == 0:
            n = int(np.prod(self.dimension))
            H = sparse.csr_matrix((n, n), dtype=complex)
        else:
            H = sparse.csr_matrix(self.hamiltonian_matrix())
        return Hamiltonian(H, dim=self.dimension)

    @property
    def lindbladian(self):
        """Lindbladian of the Hamiltonian and the dissipation terms
        (muspinsim/spinsys.py:628-634); propagated on the GPU."""
        from muspinsim_gb300.lindbladian import Lindbladian

        return Lindbladian.from_hamiltonian(self.hamiltonian,
                                            [t.tuple for t in self._dissip_terms])

    def zeeman_operators(self):
        """Z_a = sum_i gamma_i S^a_i (dense, a = x, y, z): Hz(B) = sum_a B_a Z_a
        (muspinsim/experiment.py:105-111, 239-250)."""

        def build():
            n = int(np.prod(self.dimension))
            Z = np.zeros((3, n, n), dtype=complex)
            for i in range(len(self)):
                for a, ax in enumerate("xyz"):
                    Z[a] += self._gammas[i] * self.operator({i: ax}).matrix.toarray()
            return Z

        key = ("Z", ())
        cache = self.__dict__.setdefault("_matrix_cache", {})
        if key not in cache:
            cache[key] = build()
        return cache[key].copy()

    def rotation_basis(self):
        """Term tensors and operator basis of the tensor-rotation assembly
        (msp_assemble_rotated): ``(tensors (Kd, 3, 3), vectors (Ks, 3),
        basis (9 Kd + 3 Ks, n, n) complex)`` with, per bilinear term, the
        nine Kronecker-embedded S^a_i S^b_j (the product S^a_i S^b_i for a
        same-spin term) and, per single term, the three S^a_i -- the same
        operators _recalc_operator sums (muspinsim/spinsys.py:34-69)."""
        doubles = [t for t in self._terms if isinstance(t, DoubleTerm)]
        singles = [t for t in self._terms if isinstance(t, SingleTerm)]
        if len(doubles) + len(singles) != len(self._terms):
            raise ValueError("rotation_basis: only single and double terms can be rotated")

        def dense(op):
            m = op.matrix
            return m.toarray() if sparse.issparse(m) else np.asarray(m)

        basis = []
        for t in doubles:
            i, j = int(t.i), int(t.j)
            for a in "xyz":
                for b in "xyz":
                    spec = {i: [a, b]} if i == j else {i: a, j: b}
                    basis.append(dense(self.operator(spec)))
        for t in singles:
            for a in "xyz":
                basis.append(dense(self.operator({int(t.i): a})))
        n = int(np.prod(self.dimension))
        tensors = np.array([t.tensor for t in doubles], dtype=float).reshape(-1, 3, 3)
        vectors = np.array([t.tensor for t in singles], dtype=float).reshape(-1, 3)
        B = np.array(basis, dtype=complex).reshape(-1, n, n)
        return tensors, vectors, B

    def device_matrices(self, device):
        """(Hsys, Z) as complex128 torch tensors on ``device``, uploaded once
        per term list and device (the batched GPU paths reuse them)."""
        import torch

        key = ("device", tuple(id(t) for t in self._terms), str(device))
        cache = self.__dict__.setdefault("_matrix_cache", {})
        if key not in cache:
            cache[key] = (torch.as_tensor(self.hamiltonian_matrix()).to(device),
                          torch.as_tensor(self.zeeman_operators()).to(device))
        return cache[key]

    def __len__(self):
        return len(self._gammas)


class MuonSpinSystem(SpinSystem):
    """Spin system with exactly one muon (muspinsim/spinsys.py:640-760)."""

    def __init__(self, spins=["mu", "e"], celio_k=0):
        super(MuonSpinSystem, self).__init__(spins, celio_k)
        if self._spins.count("mu") != 1:
            raise ValueError("Spins passed to MuonSpinSystem must contain exactly one muon")
        self._mu_i = self._spins.index("mu")
        self._e_i = set([i for i, s in enumerate(self.spins) if s == "e"])
        self._mu_ops = None

    @property
    def muon_index(self):
        return self._mu_i

    @property
    def elec_indices(self):
        return self._e_i

    def add_hyperfine_term(self, i, A, j=None):
        """S_i A S_j with j an electron (muspinsim/spinsys.py:664-705)."""
        elec_i = self.elec_indices
        if j is None:
            if len(elec_i) > 1:
                raise ValueError("Must specify an electron index in system with multiple electrons")
            j = list(elec_i)[0]
        else:
            if j not in elec_i:
                raise ValueError("Second index in hyperfine coupling must refer to an electron")
        if i in elec_i:
            raise ValueError("First index in hyperfine coupling must not refer to an electron")
        logging.info("Adding hyperfine term to spins %s-%s", i + 1, j + 1)
        return self.add_bilinear_term(i, j, A, "Hyperfine")

    def muon_operator(self, v):
        """sum_a v_a S^a_mu (muspinsim/spinsys.py:707-732)."""
        if len(v) != 3:
            raise ValueError("Vector passed to muon_operator must be three dimensional")
        if self._mu_ops is None:
            self._mu_ops = [self.operator({self._mu_i: e}) for e in "xyz"]
        op = [x * self._mu_ops[i] for i, x in enumerate(v)]
        return sum(op[1:], op[0])

    def sigma_mu(self, v):
        """sum_a v_a sigma_a, the 2x2 Pauli combination as CSR
        (muspinsim/spinsys.py:734-760)."""
        if len(v) != 3:
            raise ValueError("Vector passed to muon_operator must be three dimensional")
        paulis = [
            sparse.csr_matrix(np.array([[0, 1], [1, 0]], dtype=complex)),
            sparse.csr_matrix(np.array([[0, -1j], [1j, 0]], dtype=complex)),
            sparse.csr_matrix(np.array([[1, 0], [0, -1]], dtype=complex)),
        ]
        return np.sum([x * paulis[i] for i, x in enumerate(v)])
