"""Host-side logic of the MANEIG wrappers (no GPU)."""
import numpy as np

from grasp_gb300.core import rci_select_ivec


def test_rci_ivec_selection_follows_the_swap_loop():
    """rci90/maneig.f90:496-516: IVEC = (2, 4) out of the lowest 4 states
    gives states 2 and 4; IVEC = (1, 2, 3) leaves the order. The loop swaps
    positions, so a descending IVEC = (3, 1) gives what the reference gives:
    i = 1 swaps positions 3 and 1 (states 3, 2, 1), i = 2 swaps positions 1
    and 2 (states 2, 3, 1), and the first two are kept."""
    ev = np.array([-3.0, -2.0, -1.5, -1.0])
    vec = np.arange(12.0).reshape(3, 4)
    e, v = rci_select_ivec(ev, vec, [2, 4])
    np.testing.assert_array_equal(e, [-2.0, -1.0])
    np.testing.assert_array_equal(v, vec[:, [1, 3]])
    e, v = rci_select_ivec(ev[:3], vec[:, :3], [3, 1])
    np.testing.assert_array_equal(e, [-2.0, -1.5])
    np.testing.assert_array_equal(v, vec[:, [1, 2]])
    e, v = rci_select_ivec(ev[:3], vec[:, :3], [1, 2, 3])
    np.testing.assert_array_equal(e, ev[:3])
