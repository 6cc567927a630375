"""MeasurementSet input for the v4 arrays.

``MeasurementSetLoader(msfile, auto_correlations=False)`` has the interface
and semantics of the reference's loaders
(``montblanc/impl/common/loaders/loaders.py:35-137`` for opening the tables
and the problem dimensions, ``montblanc/impl/rime/v4/loaders/loaders.py:
49-246`` for ``load``):

* rows of field 0, without auto-correlations unless asked for, ordered by
  time, antenna 1, antenna 2 and spectral window (the reference's TaQL
  ``ORDERBY TIME, ANTENNA1, ANTENNA2, [SPECTRAL_WINDOW_ID][DATA_DESC_ID]``);
* ntime = distinct times, nbl = distinct antenna pairs, na = rows of the
  ANTENNA table, nbands = rows of SPECTRAL_WINDOW, nchan = the sum of their
  NUM_CHAN, which must all be equal;
* frequency = CHAN_FREQ of every band, ref_frequency = each band's
  REF_FREQUENCY repeated over its channels;
* per-antenna uvw with antenna 0 at the origin and antenna k at the UVW of
  baseline (0, k) (so baseline uvw = uvw[antenna2] - uvw[antenna1] holds for
  consistent data), from the rows of distinct (time, antenna1, antenna2);
* antenna1 / antenna2 as (ntime, nbl);
* parallactic angles of the field-0 phase centre (right ascension taken
  into [0, 2 pi)) from the ANTENNA positions at the distinct times;
* observed_vis from DATA, flag = FLAG or FLAG_ROW, and, per the solver
  configuration's ``init_weights``: weight_vector from WEIGHT_SPECTRUM,
  else WEIGHT repeated over channels ('weight'), from SIGMA_SPECTRUM, else
  SIGMA ('sigma', used as the weight as the reference does), else ones.

``msfile`` is the path of a MeasurementSet, read through python-casacore
(``casacore.tables`` or ``pyrap.tables``), or a mapping {table name:
{column name: array}} holding the MAIN, ANTENNA, SPECTRAL_WINDOW, FIELD and
DATA_DESCRIPTION tables in memory.  The row selection and ordering are done
with NumPy on whole columns, so the main table's selected columns are held
in host memory once.
"""
import logging
import math
from collections.abc import Mapping

import numpy as np

from .config import Options

log = logging.getLogger('montblanc_gb300')

MAIN = 'MAIN'
ANTENNA = 'ANTENNA'
SPECTRAL_WINDOW = 'SPECTRAL_WINDOW'
FIELD = 'FIELD'
DATA_DESCRIPTION = 'DATA_DESCRIPTION'
SUBTABLES = (ANTENNA, SPECTRAL_WINDOW, FIELD, DATA_DESCRIPTION)

INIT_WEIGHTS_NONE = None
INIT_WEIGHTS_SIGMA = 'sigma'
INIT_WEIGHTS_WEIGHT = 'weight'
VALID_INIT_WEIGHTS = (INIT_WEIGHTS_NONE, INIT_WEIGHTS_SIGMA, INIT_WEIGHTS_WEIGHT)


class MemoryTable(object):
    """A table as a mapping of column name -> array (first axis = rows)."""

    def __init__(self, columns):
        self._cols = {k: np.asarray(v) for k, v in columns.items()}
        sizes = set(len(v) for v in self._cols.values())
        if len(sizes) > 1:
            raise ValueError('table columns have different row counts %s' % sorted(sizes))
        self._nrows = sizes.pop() if sizes else 0

    def colnames(self):
        return list(self._cols)

    def getcol(self, name):
        if name not in self._cols:
            raise KeyError('no column %s' % name)
        return self._cols[name]

    def nrows(self):
        return self._nrows

    def close(self):
        pass


class _CasacoreTable(object):
    def __init__(self, tables_module, path):
        self._t = tables_module.table(path, ack=False, readonly=True)

    def colnames(self):
        return list(self._t.colnames())

    def getcol(self, name):
        return np.asarray(self._t.getcol(name))

    def nrows(self):
        return int(self._t.nrows())

    def close(self):
        self._t.close()


def open_tables(msfile):
    """{table name: table} for a MeasurementSet path or an in-memory mapping."""
    if isinstance(msfile, Mapping):
        missing = [n for n in (MAIN,) + SUBTABLES if n not in msfile]
        if missing:
            raise KeyError('in-memory MeasurementSet lacks tables %s' % missing)
        return {n: t if hasattr(t, 'getcol') else MemoryTable(t) for n, t in msfile.items()}
    try:
        from casacore import tables as tmod
    except ImportError:
        try:
            import pyrap.tables as tmod
        except ImportError:
            raise ImportError('reading the MeasurementSet %s needs python-casacore (casacore.tables), which '
                              'is not installed; pass the tables as a mapping {name: {column: array}} '
                              'instead' % msfile)
    out = {MAIN: _CasacoreTable(tmod, msfile)}
    for n in SUBTABLES:
        out[n] = _CasacoreTable(tmod, '::'.join((msfile, n)))
    return out


def _distinct_rows(*keys):
    """Mask of the rows (already ordered by keys) that start a new key tuple."""
    n = len(keys[0])
    first = np.zeros(n, dtype=bool)
    if n:
        first[0] = True
        for k in keys:
            first[1:] |= k[1:] != k[:-1]
    return first


class MeasurementSetLoader(object):
    LOG_PREFIX = 'LOADER:'

    def __init__(self, msfile, auto_correlations=False):
        self.msfile = msfile
        self.tables = open_tables(msfile)
        main = self.tables[MAIN]
        field = main.getcol('FIELD_ID')
        a1, a2 = main.getcol('ANTENNA1'), main.getcol('ANTENNA2')
        time = main.getcol('TIME')
        spw_of_ddid = self.tables[DATA_DESCRIPTION].getcol('SPECTRAL_WINDOW_ID')
        spw = spw_of_ddid[main.getcol('DATA_DESC_ID')]
        keep = field == 0  # the field is fixed at 0, as in the reference
        if not auto_correlations:
            keep &= a1 != a2
        rows = np.flatnonzero(keep)
        order = np.lexsort((spw[rows], a2[rows], a1[rows], time[rows]))
        self.rows = rows[order]
        self.auto_correlations = bool(auto_correlations)

        t, p, q = time[self.rows], a1[self.rows], a2[self.rows]
        self.nrows = len(self.rows)
        self.na = self.tables[ANTENNA].nrows()
        self.ntime = int(_distinct_rows(t).sum())
        self.nbl = len(set(zip(p.tolist(), q.tolist())))
        chan_per_band = np.asarray(self.tables[SPECTRAL_WINDOW].getcol('NUM_CHAN'))
        if not np.all(chan_per_band == chan_per_band[0]):
            raise ValueError('Channels per band %s are not equal!' % chan_per_band.tolist())
        self.nbands = len(chan_per_band)
        self.nchan = int(chan_per_band.sum())
        self._log('Found %d antenna(s), %d time(s), %d baseline(s), %d band(s) of %d channel(s)'
                  % (self.na, self.ntime, self.nbl, self.nbands, int(chan_per_band[0])))
        if self.ntime * self.nbl * self.nbands != self.nrows:
            log.warning('%s %d x %d x %d = %d does not equal the number of selected rows %d', self.LOG_PREFIX,
                        self.ntime, self.nbl, self.nbands, self.ntime * self.nbl * self.nbands, self.nrows)

    def _log(self, msg):
        log.info('%s %s', self.LOG_PREFIX, msg)

    def get_dims(self):
        """(ntime, nbl, na, nbands, nchan)"""
        return self.ntime, self.nbl, self.na, self.nbands, self.nchan

    def column(self, name):
        """Column ``name`` of the selected main-table rows, in load order."""
        return np.asarray(self.tables[MAIN].getcol(name))[self.rows]

    def has_column(self, name):
        return name in self.tables[MAIN].colnames()

    # ---- the v4 arrays ---------------------------------------------------
    def arrays(self, init_weights=INIT_WEIGHTS_NONE):
        """The v4 arrays of the MeasurementSet as float64 / complex128 /
        int32 / uint8 NumPy arrays (weight_vector only with init_weights)."""
        if init_weights not in VALID_INIT_WEIGHTS:
            raise ValueError('init_weights %r is not one of %r' % (init_weights, VALID_INIT_WEIGHTS))
        ntime, nbl, na, nbands, nchan = self.get_dims()
        out = {}
        sw = self.tables[SPECTRAL_WINDOW]
        out['frequency'] = np.asarray(sw.getcol('CHAN_FREQ'), dtype=np.float64).reshape(nchan)
        out['ref_frequency'] = np.repeat(np.asarray(sw.getcol('REF_FREQUENCY'), dtype=np.float64),
                                         np.asarray(sw.getcol('NUM_CHAN')))

        # one row per (time, antenna1, antenna2): the first band's
        time, p, q = self.column('TIME'), self.column('ANTENNA1'), self.column('ANTENNA2')
        first = _distinct_rows(time, p, q)
        bl_uvw = self.column('UVW')[first]
        if bl_uvw.shape != (ntime * nbl, 3):
            raise ValueError('MS UVW shape %s != expected %s' % (bl_uvw.shape, (ntime * nbl, 3)))
        uvw = np.zeros((ntime, na, 3), dtype=np.float64)
        # baselines (0, 1) .. (0, na - 1) come first in each time's ordering
        uvw[:, 1:na, :] = bl_uvw.reshape(ntime, nbl, 3)[:, :na - 1, :]
        out['uvw'] = uvw
        out['antenna1'] = p[first].reshape(ntime, nbl).astype(np.int32)
        out['antenna2'] = q[first].reshape(ntime, nbl).astype(np.int32)

        from .util import parallactic_angles
        times = time[_distinct_rows(time)]
        positions = np.asarray(self.tables[ANTENNA].getcol('POSITION'), dtype=np.float64)
        phase_dir = np.array(np.asarray(self.tables[FIELD].getcol('PHASE_DIR'), dtype=np.float64)[0][0])
        if phase_dir[0] < 0:
            phase_dir[0] += 2 * math.pi
        out['parallactic_angles'] = parallactic_angles(phase_dir, positions, times)

        vshape = (ntime, nbl, nchan, 4)
        if self.has_column('DATA'):
            self._log('Loading visibilities into the observed_vis array')
            out['observed_vis'] = self.column('DATA').astype(np.complex128).reshape(vshape)
        if self.has_column('FLAG'):
            self._log('Loading flag data')
            flag = self.column('FLAG').astype(bool)
            if self.has_column('FLAG_ROW'):
                flag = flag | self.column('FLAG_ROW').astype(bool)[:, None, None]
            out['flag'] = flag.reshape(vshape).astype(np.uint8)

        if init_weights is not INIT_WEIGHTS_NONE:
            spectrum, plain = (('WEIGHT_SPECTRUM', 'WEIGHT') if init_weights == INIT_WEIGHTS_WEIGHT
                               else ('SIGMA_SPECTRUM', 'SIGMA'))
            cpb = nchan // nbands
            if self.has_column(spectrum):
                self._log('Initialising weight_vector from %s' % spectrum)
                wv = self.column(spectrum).astype(np.float64)
            elif self.has_column(plain):
                self._log('Initialising weight_vector from %s' % plain)
                wv = np.repeat(self.column(plain).astype(np.float64)[:, None, :], cpb, axis=1)
            else:
                self._log('No %s or %s column: weight_vector set to ones' % (spectrum, plain))
                wv = np.ones((ntime * nbl * nbands, cpb, 4))
            if wv.shape != (ntime * nbl * nbands, cpb, 4):
                raise ValueError('weight shape %s != expected %s' % (wv.shape, (ntime * nbl * nbands, cpb, 4)))
            out['weight_vector'] = wv.reshape(vshape)
        return out

    def load(self, solver, slvr_cfg):
        """Transfer the MeasurementSet's arrays into ``solver`` (any object
        with ``transfer_<array>`` methods, cast to its array dtypes)."""
        arrs = self.arrays(slvr_cfg.get(Options.INIT_WEIGHTS, INIT_WEIGHTS_NONE))
        for name, a in arrs.items():
            getattr(solver, 'transfer_' + name)(np.ascontiguousarray(a))

    def close(self):
        for t in self.tables.values():
            t.close()

    def __enter__(self):
        return self

    def __exit__(self, exc_type, exc, tb):
        self.close()
        return False
