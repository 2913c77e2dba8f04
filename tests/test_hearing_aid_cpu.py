"""The hearing-aid restatement on small cases worked by hand."""
import numpy as np

from oracle import oracle as orc


def test_hand_cases():
    x = np.array([[1.0, 2.0, 3.0, 4.0]], np.float32)
    # FIR [1]: the first sample gets no term (bound min(n, L)), the rest pass
    out = orc.hearing_aid(x, np.ones(1, np.float32), np.zeros(0, np.float32))
    assert out.tolist() == [[0.0, 2.0, 3.0, 4.0]]
    # FIR [1, 0.5]: aux = [0, 2, 3+1, 4+1.5]
    out = orc.hearing_aid(x, np.array([1.0, 0.5], np.float32), np.zeros(0, np.float32))
    assert out.tolist() == [[0.0, 2.0, 4.0, 5.5]]
    # then out[n] = aux[n] + 0.25 aux[n-1] (the second stage reads aux)
    out = orc.hearing_aid(x, np.array([1.0, 0.5], np.float32), np.array([1.0, 0.25], np.float32))
    assert out.tolist() == [[0.0, 2.0, 4.5, 6.5]]
