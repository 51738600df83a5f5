# The Python example of the integration guide (quoted there): the reference's
# quantum_computer example loop (examples/quantum_computer_test.cpp) through
# the package's names.
import quids_gb300 as quids
from quids_gb300 import rules

quids.tolerance = 1e-18
ctx = quids.Context(0)
it, nxt, sy = quids.it_t(ctx), quids.it_t(ctx), quids.sy_it_t()
it.append(bytes(12), 1 + 0j)
quids.simulate(it, rules.hadamard(0), nxt, sy, 1 << 22)
quids.simulate(nxt, rules.Zgate(0))
print(nxt.num_object, nxt.total_proba, sy.num_object, sy.num_object_after_interferences)
