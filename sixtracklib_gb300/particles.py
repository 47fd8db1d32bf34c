"""NS(Particles): the 21-column particle SoA and its CObjects encoding.

Field order and types follow sixtracklib/common/particles.h:38-67 (17 float64
columns, then particle_id, at_element_id, at_turn, state as int64).  In a
CObjects buffer a Particles object (type id 1) is ``num_particles`` followed
by 21 column pointers and the 21 columns.  Python names follow
python/sixtracklib/particles.py (``at_element`` for ``at_element_id``).

The "column block" used throughout this package (and by the C ABI's
``st_ParticlesColumns`` helpers and the oracle) is the same 21 columns laid
out contiguously: column ``c`` occupies words ``[c*n, (c+1)*n)``.
"""

from __future__ import annotations

import numpy as np

from .cbuffer import CBuffer, CObject

REAL_FIELDS = (
    "q0", "mass0", "beta0", "gamma0", "p0c", "s", "x", "y", "px", "py",
    "zeta", "psigma", "delta", "rpp", "rvv", "chi", "charge_ratio",
)
INT_FIELDS = ("particle_id", "at_element", "at_turn", "state")
FIELDS = REAL_FIELDS + INT_FIELDS
NUM_COLUMNS = 21
COL = {name: i for i, name in enumerate(FIELDS)}
TYPE_PARTICLE = 1
PROTON_MASS_EV = 938272088.16  # internal/physics_constants.h:53


class Particles:
    """A particle set backed by one contiguous column block.

    ``Particles(num_particles=n, **columns)`` creates a fresh set with the
    reference's column defaults (python/sixtracklib/particles.py:24-192:
    mass0 = ``pmass``, beta0 = gamma0 = p0c = 1, rpp = rvv = chi =
    charge_ratio = state = 1, the rest 0) except particle_id, which is
    0..n-1 here (0 in the reference, whose ``from_ref`` numbers them), then
    any column given by name (a scalar or n values; ``at_element_id`` is an
    alias of ``at_element``).  Pass ``cbuffer=`` to append it to a CObjects
    buffer, in which case the columns live inside the buffer object and
    edits are visible to whoever serialises the buffer.
    """

    pmass = 938.2720813e6  # the reference's Python default (particles.py:23)

    def __init__(self, num_particles=0, cbuffer=None, _words=None, _index=None, **columns):
        unknown = set(columns) - set(FIELDS) - {"at_element_id"}
        if unknown:
            raise TypeError(f"Particles: unknown column(s) {sorted(unknown)}")
        n = int(num_particles)
        self.num_particles = n
        if _words is None:
            words = np.zeros(22 + NUM_COLUMNS * n, dtype=np.uint64)
            words[0] = n
            for c in range(NUM_COLUMNS):
                words[1 + c] = 22 + c * n
            self._words = words
            self._init_defaults()
        else:
            self._words = _words
        for name, value in columns.items():
            self.column("at_element" if name == "at_element_id" else name)[:] = value
        self._cbuffer = None
        self._index = _index
        if cbuffer is not None:
            obj = CObject(TYPE_PARTICLE, self._words, list(range(1, 22)))
            cbuffer.objects.append(obj)
            cbuffer.touch()
            cbuffer.typeids[TYPE_PARTICLE] = Particles
            self._index = cbuffer.n_objects - 1
            self._cbuffer = cbuffer

    def _init_defaults(self):
        n = self.num_particles
        self.mass0[:] = self.pmass
        self.beta0[:] = 1.0
        self.gamma0[:] = 1.0
        self.p0c[:] = 1.0
        self.chi[:] = 1.0
        self.charge_ratio[:] = 1.0
        self.state[:] = 1
        self.particle_id[:] = np.arange(n)
        self.rpp[:] = 1.0
        self.rvv[:] = 1.0

    # --------------------------------------------------------- columns
    def column(self, name_or_idx) -> np.ndarray:
        c = COL[name_or_idx] if isinstance(name_or_idx, str) else int(name_or_idx)
        off = int(self._words[1 + c])
        seg = self._words[off : off + self.num_particles]
        return seg.view(np.float64) if c < 17 else seg.view(np.int64)

    @property
    def block(self) -> np.ndarray:
        """The 21 x n column block as u64 words (a view when contiguous)."""
        n = self.num_particles
        offs = [int(self._words[1 + c]) for c in range(NUM_COLUMNS)]
        if offs == [22 + c * n for c in range(NUM_COLUMNS)]:
            return self._words[22 : 22 + NUM_COLUMNS * n].reshape(NUM_COLUMNS, n)
        return np.stack([self._words[o : o + n] for o in offs])

    def set_block(self, block: np.ndarray):
        block = np.asarray(block).reshape(NUM_COLUMNS, -1).view(np.uint64)
        for c in range(NUM_COLUMNS):
            off = int(self._words[1 + c])
            self._words[off : off + self.num_particles] = block[c]
        if self._cbuffer is not None:
            self._cbuffer.touch()

    def copy(self) -> "Particles":
        p = Particles(self.num_particles)
        p.set_block(self.block.copy())
        return p

    # --------------------------------------------------------- physics
    def set_reference(self, p0c=7e12, mass0=pmass, q0=1.0):
        """Reference momentum, mass and charge; beta0/gamma0 from p0c (the
        reference sets q0, mass0 and p0c only and leaves beta0, gamma0 as
        they were)."""
        energy0 = np.sqrt(p0c * p0c + mass0 * mass0)
        self.q0[:] = q0
        self.mass0[:] = mass0
        self.p0c[:] = p0c
        self.beta0[:] = p0c / energy0
        self.gamma0[:] = energy0 / mass0
        return self

    def set_delta(self, delta):
        """Set delta and the dependent rvv, rpp, psigma with the arithmetic of
        NS(Particles_update_delta_value) (particles.h:5459-5496)."""
        d = np.asarray(delta, dtype=np.float64) * np.ones(self.num_particles)
        beta0 = self.beta0.copy()
        delta_beta0 = d * beta0
        ptau_beta0 = np.sqrt(delta_beta0 * delta_beta0 + 2.0 * delta_beta0 * beta0 + 1.0) - 1.0
        opd = 1.0 + d
        self.delta[:] = d
        self.rvv[:] = opd / (1.0 + ptau_beta0)
        self.rpp[:] = 1.0 / opd
        self.psigma[:] = ptau_beta0 / (beta0 * beta0)
        return self

    @classmethod
    def from_ref(cls, num_particles=1, mass0=pmass, p0c=1e9, q0=1.0):
        return cls(num_particles=num_particles).set_reference(p0c=p0c, mass0=mass0, q0=q0)

    # the reference's derived quantities (particles.py:202-208)
    @property
    def ptau(self):
        return np.sqrt(self.delta ** 2 + 2 * self.delta + 1 / self.beta0 ** 2) - 1 / self.beta0

    @property
    def beta(self):
        return (1 + self.delta) / (1 / self.beta0 + self.ptau)

    @property
    def sigma(self):
        return (self.beta0 / self.beta) * self.zeta

    # one particle to / from a pysixtrack Particles (particles.py:216-270)
    _PYSIX = (("q0", "q0"), ("mass0", "mass0"), ("beta0", "beta0"), ("gamma0", "gamma0"),
              ("p0c", "p0c"), ("s", "s"), ("x", "x"), ("y", "y"), ("px", "px"), ("py", "py"),
              ("zeta", "zeta"), ("psigma", "psigma"), ("delta", "delta"), ("chi", "chi"),
              ("charge_ratio", "qratio"), ("at_element", "elemid"), ("at_turn", "turn"),
              ("state", "state"))

    def from_pysixtrack(self, inp, particle_index):
        assert particle_index < self.num_particles
        for mine, theirs in self._PYSIX:
            getattr(self, mine)[particle_index] = getattr(inp, theirs)
        self.rpp[particle_index] = inp.rpp
        self.rvv[particle_index] = inp.rvv
        pid = getattr(inp, "partid", None)
        self.particle_id[particle_index] = pid if pid is not None else particle_index
        if self._cbuffer is not None:
            self._cbuffer.touch()

    def to_pysixtrack(self, other, particle_index):
        """Write particle ``particle_index`` into ``other`` with its
        coordinate update suspended, as the reference does."""
        assert particle_index < self.num_particles
        other._update_coordinates = False
        for mine, theirs in self._PYSIX:
            setattr(other, theirs, getattr(self, mine)[particle_index])
        other.partid = self.particle_id[particle_index]
        other._update_coordinates = True

    @classmethod
    def _from_cobject(cls, obj: CObject, cbuffer=None, index=None):
        n = int(obj.words[0])
        p = cls(num_particles=n, _words=obj.words, _index=index)
        p._cbuffer = cbuffer
        return p

    def __len__(self):
        return self.num_particles


def _make_prop(name):
    def getter(self):
        return self.column(name)

    def setter(self, value):
        self.column(name)[:] = value
        if self._cbuffer is not None:
            self._cbuffer.touch()

    return property(getter, setter)


for _name in FIELDS:
    setattr(Particles, _name, _make_prop(_name))
Particles.at_element_id = _make_prop("at_element")


def makeCopy(orig, cbuffer=None):
    """A new particle set with the columns of ``orig`` (particles.py:292-320)."""
    return Particles(num_particles=orig.num_particles, cbuffer=cbuffer,
                     **{name: getattr(orig, name) for name in FIELDS})


def calcParticlesDifference(lhs, rhs, cbuffer=None):
    """Column-wise lhs - rhs as a particle set (particles.py:323-358)."""
    assert lhs.num_particles == rhs.num_particles
    diff = Particles(num_particles=lhs.num_particles, cbuffer=cbuffer)
    for name in FIELDS:
        diff.column(name)[:] = getattr(lhs, name) - getattr(rhs, name)
    return diff


def compareParticlesDifference(lhs, rhs, abs_treshold=None):
    """0 when the sets agree, else the sign of the first differing entry
    (lhs > rhs: +1), columns in order, float columns first; with
    ``abs_treshold`` > 0 float entries differing by no more than it count as
    equal; -1 for different or zero particle counts (particles.py:361-415)."""
    n = lhs.num_particles
    if n != rhs.num_particles or n <= 0:
        return -1
    tol = abs_treshold if abs_treshold is not None and abs_treshold > 0.0 else None
    for names, use_tol in ((REAL_FIELDS, True), (INT_FIELDS, False)):
        for name in names:
            a, b = getattr(lhs, name), getattr(rhs, name)
            if np.array_equal(a, b):
                continue
            if use_tol and tol is not None:
                bad = np.nonzero(np.abs(a - b) > tol)[0]
            else:  # NaN compares neither greater nor smaller
                bad = np.nonzero((a > b) | (a < b))[0]
            if bad.size:
                i = bad[0]
                return +1 if a[i] > b[i] else -1
    return 0


TYPE_PARTICLES_ADDR = 512


def _particles_addr_class():
    from .beam_elements import _Element

    class ParticlesAddr(_Element):
        """NS(ParticlesAddr) as a buffer object (particles.py:490-513, type
        id 512): the particle count and the address of each of the 21
        columns, in NS(Particles) order."""

        _typeid = TYPE_PARTICLES_ADDR
        _fields = (("num_particles", "i"),) + tuple(
            (name, "u") for name in (
                "q0", "mass0", "beta0", "gamma0", "p0c", "s", "x", "y", "px", "py", "zeta",
                "psigma", "delta", "rpp", "rvv", "chi", "charge_ratio", "particle_id",
                "at_element", "at_turn", "state"))

    return ParticlesAddr


ParticlesAddr = _particles_addr_class()


class ParticlesSet:
    """Container of particle sets in one CObjects buffer
    (python/sixtracklib/particles.py:417-489)."""

    def __init__(self, cbuffer=None):
        self.cbuffer = CBuffer() if cbuffer is None else cbuffer
        self.cbuffer.typeids[TYPE_PARTICLE] = Particles

    def Particles(self, num_particles=0, **kw):
        return Particles(num_particles=num_particles, cbuffer=self.cbuffer, **kw)

    @property
    def particles(self):
        return [self.cbuffer.get_object(i) for i in range(self.cbuffer.n_objects)
                if self.cbuffer.objects[i].typeid == TYPE_PARTICLE]

    @classmethod
    def fromSixDump101(cls, input_folder, st_dump_file, **kwargs):
        """Particle sets from a SixTrack DUMP format-101 file, one set per
        dump location (particles.py:443-488).  Like the reference this needs
        sixtracktools and pysixtrack to read the SixTrack input and the dump;
        it raises ImportError where they are not installed."""
        import pysixtrack
        import sixtracktools

        six = sixtracktools.SixInput(input_folder)
        line, rest, iconv = six.expand_struct(convert=pysixtrack.element_types)
        sixdump = sixtracktools.SixDump101(st_dump_file)
        num_iconv, num_belem, num_dumps = len(iconv), len(line), len(sixdump.particles)
        if not (num_iconv > 0 and num_belem > iconv[-1] and num_dumps >= num_iconv and
                num_dumps % num_iconv == 0):
            raise ValueError("SixTrack dump and input do not match")
        n = num_dumps // num_iconv
        self = cls(**kwargs)
        for ii, elem_id in enumerate(iconv):
            p = self.Particles(num_particles=n)
            for jj in range(n):
                p.from_pysixtrack(pysixtrack.Particles(**sixdump[n * ii + jj].get_minimal_beam()),
                                  jj)
                p.state[jj] = 1
                p.at_element[jj] = elem_id
        return self

    @classmethod
    def fromfile(cls, filename):
        return cls(cbuffer=CBuffer.fromfile(filename))

    def to_file(self, filename):
        self.cbuffer.tofile(filename)
        return self
