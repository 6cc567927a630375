"""Pipeline node interface (montblanc/node.py:21-139).

A node is one stage of a RIME pipeline.  The solver calls, for every node,
``initialise`` once, then ``pre_execution`` / ``execute`` / ``post_execution``
per solve, and ``shutdown`` at the end.  ``stream`` is a ``torch.cuda.Stream``
(or None for the current stream); GPU nodes launch on it.
"""


class Node(object):
    def __init__(self):
        pass

    def description(self):
        """Name of the node, used in logging."""
        return self.__class__.__name__

    def initialise(self, solver, stream=None):
        raise NotImplementedError(self._missing('initialise'))

    def shutdown(self, solver, stream=None):
        raise NotImplementedError(self._missing('shutdown'))

    def pre_execution(self, solver, stream=None):
        raise NotImplementedError(self._missing('pre_execution'))

    def execute(self, solver, stream=None):
        raise NotImplementedError(self._missing('execute'))

    def post_execution(self, solver, stream=None):
        raise NotImplementedError(self._missing('post_execution'))

    def _missing(self, fn):
        return 'method %s not implemented in class %s derived from abstract class Node' % (
            fn, type(self).__name__)


class NullNode(Node):
    """A node that does nothing."""

    def initialise(self, solver, stream=None):
        pass

    def shutdown(self, solver, stream=None):
        pass

    def pre_execution(self, solver, stream=None):
        pass

    def execute(self, solver, stream=None):
        pass

    def post_execution(self, solver, stream=None):
        pass
