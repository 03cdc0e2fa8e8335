"""hmf_data_term and hmf_log_likelihood against the oracle's restatement
(oracle/dataterm_oracle.py).  Both compute in the reference's precision and
order; CUDA's double exp / log and numpy's may differ in the last bit of the
double, which after rounding to float shows as at most one or two float ulps
in a small fraction of voxels: the tests require <= 2 ulps everywhere and
>= 99.9 % of values bit-identical (exact where no exp / log is involved).
GPU only."""
import numpy as np
import pytest

from oracle import dataterm_oracle as DT
from robartsvtk_gb300 import HMFError, ImageDataTerm, ImageLogLikelihood, data_term, log_likelihood

pytestmark = pytest.mark.gpu


def assert_ulps(got, want, max_ulps=2, exact_frac=0.999):
    got = np.asarray(got, np.float32).reshape(-1)
    want = np.asarray(want, np.float32).reshape(-1)
    gi = got.view(np.int32).astype(np.int64)
    wi = want.view(np.int32).astype(np.int64)
    gi = np.where(gi < 0, -(gi & 0x7fffffff), gi)
    wi = np.where(wi < 0, -(wi & 0x7fffffff), wi)
    d = np.abs(gi - wi)
    assert d.max() <= max_ulps, "max %d ulps" % d.max()
    assert (d == 0).mean() >= exact_frac, "only %.5f exact" % (d == 0).mean()


def image(seed, shape=(23, 17, 11), lo=-3.0, hi=5.0):
    rng = np.random.default_rng(seed)
    return rng.uniform(lo, hi, size=shape).astype(np.float32)


CONSTS = dict(k1=1.7, c1=0.6, k2=0.8, c2=-0.4)


@pytest.mark.parametrize("op", [DT.CONSTANT, DT.LOGISTIC, DT.GAUSSIAN, DT.SPIKE])
@pytest.mark.parametrize("entropy", [False, True])
@pytest.mark.parametrize("normalize", [False, True])
def test_one_image(op, entropy, normalize):
    x = image(1)
    x.reshape(-1)[::7] = np.float32(1.7)  # spike hits
    c = dict(CONSTS, c1=0.6 if not (entropy and op in (DT.CONSTANT, DT.SPIKE)) else 0.35, c2=0.7)
    want = DT.data_term(op, x, entropy=entropy, normalize=normalize, **c)
    got = data_term(op, x, entropy=entropy, normalize=normalize, **c)
    assert_ulps(got, want)


@pytest.mark.parametrize("op", [DT.CONSTANT, DT.LOGISTIC, DT.GAUSSIAN])
@pytest.mark.parametrize("entropy", [False, True])
def test_two_images_host_and_device(op, entropy):
    torch = pytest.importorskip("torch")
    x1, x2 = image(2), image(3)
    c = dict(CONSTS, c1=0.3, c2=0.6)
    want = DT.data_term(op, x1, x2, entropy=entropy, **c)
    assert_ulps(data_term(op, x1, x2, entropy=entropy, **c), want)
    got = data_term(op, torch.from_numpy(x1).cuda(), torch.from_numpy(x2).cuda(), entropy=entropy, **c)
    assert got.is_cuda
    assert_ulps(got.cpu().numpy(), want)


def test_data_term_errors_and_facade():
    x = image(4)
    with pytest.raises(HMFError, match="spike"):
        data_term(DT.SPIKE, x, x)
    f = ImageDataTerm()
    f.SetInput1Data(x)
    f.SetOperationToSpike()  # the Gaussian code, as the reference
    f.SetConstantK1(2.0)
    f.SetConstantC1(0.5)
    f.SetOutputToEntropy()
    assert f.Update() == 1
    assert_ulps(f.GetOutput(), DT.data_term(DT.GAUSSIAN, x, k1=2.0, c1=0.5, entropy=True, normalize=True))


def seeds(seed, shape, n_maps, label=2):
    rng = np.random.default_rng(seed)
    truth = (rng.random(shape) < 0.3).astype(np.int32) * label
    maps = []
    for k in range(n_maps):
        m = truth.copy()
        flip = rng.random(shape) < 0.1
        m[flip] = label - m[flip]
        maps.append(m)
    return maps


@pytest.mark.parametrize("agreement,normalize", [(0.8, False), (0.5, True), (1.0, False), (0.0, True)])
def test_log_likelihood_one_component(agreement, normalize):
    shape = (31, 19, 13)
    img = np.round(image(5, shape, 0.0, 120.0))  # integral values, resolution 1
    maps = seeds(6, shape, 4) + [None]
    want = DT.log_likelihood(img, maps, label_id=2, resolution=1.0, required_agreement=agreement, normalize=normalize)
    got = log_likelihood(img, maps, label_id=2, resolution=1.0, required_agreement=agreement, normalize=normalize)
    assert_ulps(got, want)


def test_log_likelihood_two_components_and_device():
    torch = pytest.importorskip("torch")
    shape = (17, 11, 9)
    img = np.round(image(7, shape + (2,), 0.0, 40.0)).reshape(-1)
    maps = seeds(8, shape, 3, label=1)
    want = DT.log_likelihood(img, maps, label_id=1, resolution=2.0, required_agreement=0.6, components=2)
    got = log_likelihood(img, maps, label_id=1, resolution=2.0, required_agreement=0.6, components=2)
    assert_ulps(got, want)
    dev = log_likelihood(torch.from_numpy(img).cuda(), [torch.from_numpy(m.reshape(-1)).cuda() for m in maps],
                         label_id=1, resolution=2.0, required_agreement=0.6, components=2)
    assert_ulps(dev.cpu().numpy(), want)


@pytest.mark.parametrize("hi,comps", [(20000.0, 1), (199.0, 2)])
def test_log_likelihood_large_histograms(hi, comps):
    """Histograms of more bins than one CTA's shared memory holds (20001 bins;
    200 x 200) are counted with global atomics; same costs."""
    shape = (23, 17, 11)
    img = np.round(image(12, shape + ((comps,) if comps == 2 else ()), 0.0, hi)).reshape(-1)
    maps = seeds(13, shape, 3, label=1)
    want = DT.log_likelihood(img, maps, label_id=1, resolution=1.0, required_agreement=0.6, components=comps)
    got = log_likelihood(img, maps, label_id=1, resolution=1.0, required_agreement=0.6, components=comps)
    assert_ulps(got, want)


def test_log_likelihood_no_seed_overflow_and_facade():
    shape = (8, 8, 8)
    img = image(9, shape, 10.0, 20.0)
    maps = seeds(10, shape, 2)
    assert np.all(log_likelihood(img, maps, label_id=5) == 1.0)
    with pytest.raises(HMFError, match="past its histogram"):
        log_likelihood(img, maps, label_id=2, resolution=0.5, required_agreement=0.5)
    ll = ImageLogLikelihood()
    img2 = np.round(image(11, shape, 0.0, 50.0))
    ll.SetInputDataImage(img2)
    for k, m in enumerate(maps):
        ll.SetInputLabelMapData(m, k)
    ll.SetLabelID(2)
    ll.SetRequiredAgreement(0.5)
    ll.SetNormalizeDataTermOn()
    assert ll.Update() == 1
    assert_ulps(ll.GetOutput(), DT.log_likelihood(img2, maps, label_id=2, required_agreement=0.5, normalize=True))
