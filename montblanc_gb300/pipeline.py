"""Ordered list of nodes driven by a solver (montblanc/pipeline.py:29-177).

Error behaviour follows the reference: an exception raised by a node is
logged and turns the call's return value into False instead of
propagating.  The exception is kept in ``last_error`` so callers (and tests)
can inspect or re-raise it.  Unlike the reference, ``execute`` returns True
when every node succeeded (the reference returns False in both cases,
pipeline.py:137).
"""
import logging

from .node import NullNode

log = logging.getLogger('montblanc_gb300')


class PipeLineError(Exception):
    """Pipeline exception base class."""


class Pipeline(object):
    def __init__(self, node_list=None):
        if node_list is None:
            node_list = [NullNode()]
        if not isinstance(node_list, list):
            raise TypeError('node_list argument is not a list')
        self.pipeline = node_list
        self.initialised = False
        self.nr_of_executions = 0
        self.last_error = None

    def is_initialised(self):
        return self.initialised

    def _guard(self, phase, fn):
        try:
            fn()
            return True
        except Exception as e:  # noqa: BLE001 - mirrors the reference's catch-all
            self.last_error = e
            log.error('%s occurred during RIME pipeline %s',
                      'Pipeline Error' if isinstance(e, PipeLineError) else 'Unexpected exception',
                      phase, exc_info=True)
            return False

    def initialise(self, solver, stream=None):
        if self.is_initialised():
            return True

        def run():
            for node in self.pipeline:
                log.debug("Initialising node '%s'", node.description())
                node.initialise(solver, stream)

        self.initialised = self._guard('initialisation', run)
        self.nr_of_executions = 0
        return self.initialised

    def execute(self, solver, stream=None):
        if not self.is_initialised():
            log.error('Pipeline was not initialised!')
            if not self.initialise(solver, stream):
                return False

        def run():
            for node in self.pipeline:
                log.debug("Executing node '%s'", node.description())
                node.pre_execution(solver, stream)
                node.execute(solver, stream)
                node.post_execution(solver, stream)
            self.nr_of_executions += 1

        return self._guard('execution', run)

    def shutdown(self, solver, stream=None):
        ok = True
        for node in self.pipeline:
            ok = self._guard('shutdown', lambda n=node: n.shutdown(solver, stream)) and ok
        self.initialised = False
        return ok

    def __str__(self):
        return ' '.join(node.description() for node in self.pipeline)
