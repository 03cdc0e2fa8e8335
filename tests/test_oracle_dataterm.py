"""The data-term oracle (oracle/dataterm_oracle.py) on hand-checked values and
the reference's documented quirks; the facades' VTK setters.  CPU only."""
import numpy as np
import pytest

from oracle import dataterm_oracle as DT
from robartsvtk_gb300.dataterm import GAUSSIAN, SPIKE, ImageDataTerm, ImageLogLikelihood


def test_one_image_operations():
    x = np.array([0.0, 1.0, 2.0, 3.0], np.float32)
    g = DT.data_term(DT.GAUSSIAN, x, k1=1.0, c1=1.0)
    np.testing.assert_allclose(g, np.exp(-0.5 * (x - 1.0) ** 2), rtol=1e-7)
    ge = DT.data_term(DT.GAUSSIAN, x, k1=2.0, c1=1.0, entropy=True)
    np.testing.assert_allclose(ge, 0.5 * ((x - 1.0) / 2.0) ** 2, rtol=1e-7)
    lo = DT.data_term(DT.LOGISTIC, x, k1=3.0, c1=1.5)
    np.testing.assert_allclose(lo, 1.0 / (1.0 + np.exp(-3.0 * (x - 1.5))), rtol=1e-6)
    assert DT.data_term(DT.CONSTANT, x, c1=0.25).tolist() == [0.25] * 4
    np.testing.assert_allclose(DT.data_term(DT.CONSTANT, x, c1=0.25, entropy=True), -np.log(0.25), rtol=1e-7)


def test_spike_second_value_is_c1_unless_entropy():
    # vtkImageDataTerm.cxx:106: the one-image spike's "else" value is C1 ...
    x = np.array([1.0, 2.0, 5.0], np.float32)
    assert DT.data_term(DT.SPIKE, x, k1=2.0, c1=0.3, c2=0.9).tolist() == pytest.approx([0.3, 0.3, 0.3])
    # ... and -log(C2) when the output is an entropy
    e = DT.data_term(DT.SPIKE, x, k1=2.0, c1=0.3, c2=0.9, entropy=True)
    np.testing.assert_allclose(e, [-np.log(0.9), -np.log(0.3), -np.log(0.9)], rtol=1e-6)


def test_normalisation_maps_the_range_to_unit_interval():
    x = np.linspace(-2.0, 4.0, 121).astype(np.float32)  # contains c1 = 0.5
    g = DT.data_term(DT.GAUSSIAN, x, k1=1.5, c1=0.5, entropy=True, normalize=True)
    assert float(g.min()) == 0.0 and abs(float(g.max()) - 1.0) < 1e-6


def test_two_images_have_no_spike():
    x = np.zeros(3, np.float32)
    with pytest.raises(ValueError):
        DT.data_term(DT.SPIKE, x, x)


def test_log_likelihood_small_case():
    img = np.array([0, 1, 1, 2, 3, 3, 3, 9], np.float32)
    lab = np.array([1, 1, 1, 1, 1, 1, 0, 0], np.int32)
    out = DT.log_likelihood(img, [lab], label_id=1, resolution=1.0, required_agreement=1.0)
    # seeds 0,1,1,2,3,3 -> bins 0..3 with 1,2,1,2 counts of 6; 9 is past the histogram
    freq = np.array([1, 2, 1, 2], np.float64) / 6 + 1e-10
    want = [-np.log(freq[0]), -np.log(freq[1]), -np.log(freq[1]), -np.log(freq[2]), -np.log(freq[3]),
            -np.log(freq[3]), -np.log(freq[3]), -np.log(1e-10)]
    np.testing.assert_allclose(out, want, rtol=1e-6)
    assert np.all(DT.log_likelihood(img, [lab], label_id=7) == 1.0)  # no seed: cost 1


def test_log_likelihood_rejects_the_reference_overflow():
    # bins = (int)(max - min/resolution) + 1 = (int)(20 - 10/0.5) + 1 = 1, but seeds span 20 bins
    img = np.array([10.0, 20.0], np.float32)
    with pytest.raises(ValueError):
        DT.log_likelihood(img, [np.ones(2, np.int32)], resolution=0.5)


def test_facade_setters_as_the_reference():
    f = ImageDataTerm()
    assert f.GetOperation() == 0 and f.GetNormalize() is True and f.GetConstantK1() == 1.0
    f.SetOperationToGaussian()
    assert f.GetOperation() == SPIKE
    f.SetOperationToSpike()
    assert f.GetOperation() == GAUSSIAN
    ll = ImageLogLikelihood()
    assert (ll.GetLabelID(), ll.GetHistogramResolution(), ll.GetRequiredAgreement(), ll.GetNormalizeDataTerm()) == \
        (1, 1.0, 0.8, 0)
    ll.SetRequiredAgreement(3.0)
    assert ll.GetRequiredAgreement() == 1.0
