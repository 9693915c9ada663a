"""Commands: user hooks run on the host between device segments.

Mirrors ``core/command/command.py`` and ``command_sequence.py``: after each
step (after the swap) every command not yet passed whose time has come is
executed.  The model ends a device segment exactly at such a step, so a
command sees the same ``t``, ``step`` and state as in the reference.
"""


class Command:
    """A scheduled host action (core/command/command.py)."""

    def __init__(self, time=None):
        self.t = time
        self.passed = False

    def execute(self, model):
        raise NotImplementedError

    def update_status(self, model):
        self.passed = model.t >= self.t
        return self.passed


class CommandSequence:
    """Ordered commands (core/command/command_sequence.py)."""

    def __init__(self):
        self.sequence = []
        self.model = None

    def initialize(self, model):
        self.model = model
        for command in self.sequence:
            command.passed = False

    def add_command(self, command):
        self.sequence.append(command)

    def remove_commands(self):
        self.sequence = []

    def execute_next(self):
        for command in self.sequence:
            if not command.passed and command.update_status(self.model):
                command.execute(self.model)
