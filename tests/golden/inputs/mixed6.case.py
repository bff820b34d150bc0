# Six random-sequence 12-residue chains (seed 5, every residue type of the library
# can occur) at 20 mM in a periodic cube, Andersen NVT at 300 K: diverse residues,
# side-chain HB roles and several chains for the builder, the oracle and the
# engine.  The .gro text comes from the package's own generator (this script runs
# where the fixtures are made; the text is stored in the fixture).
import os as _os
import sys as _sys

_sys.path.insert(0, _os.path.dirname(_os.path.dirname(_os.path.dirname(_os.path.abspath(extra)))))
from sdmd_gb300 import workloads as _W
from sdmd_gb300.host import generate_gro as _gen

_n, _len, _mM = 6, 12, 20.0
_edge = (_n / (_mM * 1e-3 * 6.02214076e23) * 1e27) ** (1.0 / 3.0)
_d = _W._datadir(dict(temp=0.5962, thermostat="Andersen", time=1e9))
_gro = _gen(_d, _W.random_sequences(_n, _len, 5), (_edge, _edge, _edge), seed=5)

CASE = dict(gro_text=_gro, params=base_params(temp=0.5962), n_events=20000, ckpts=[5000, 10000])
