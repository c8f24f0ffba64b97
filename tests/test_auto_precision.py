"""What precision="auto" picks (host logic, no GPU): the FP64 step with the exact fixed-point exchange
sum for the models that form supports where it is faster, the all-FP64 step otherwise."""
import numpy as np

from magex_gb300.lattice import Supercell
from magex_gb300.llg import AUTO_FIXED_MIN_SITES, auto_fixed, fixed_point_eligible
from magex_gb300.spinmodel import load_results, make_model
from magex_gb300.workloads import bcc_two_site, triangular_film


def test_auto_picks_the_fixed_point_sum_for_large_tensor_stencils():
    assert auto_fixed(bcc_two_site(L=128))                      # the benchmark lattice
    assert auto_fixed(triangular_film(L=256))                   # iso + DMI film, 65,536 sites
    assert not auto_fixed(bcc_two_site(L=8))                    # 1,024 sites: latency-bound, FP64 is faster
    assert not auto_fixed(triangular_film(L=128))               # 16,384 sites
    assert AUTO_FIXED_MIN_SITES == 1 << 15


def test_auto_keeps_fp64_for_isotropic_stencils_and_unsupported_models():
    sc = Supercell(load_results(make_model("sc", J=[1.0])), (64, 64, 64))
    assert fixed_point_eligible(sc) and not auto_fixed(sc)      # width-1 couplings: FP64 gather is cheaper
    big = bcc_two_site(L=32)
    assert auto_fixed(big)
    assert not auto_fixed(big, alpha=np.full(big.N, 0.1))       # per-site damping
    assert not auto_fixed(big, sot=dict(p=[0, 1, 0], B_DL=0.1))  # spin-orbit torque
    big.mu_site = big.mu.copy()
    assert not auto_fixed(big)                                  # per-site moments
    edited = bcc_two_site(L=32)
    edited.site_T = np.full(edited.N, 300.0)
    assert not auto_fixed(edited)                               # per-site temperature


def test_auto_refuses_more_couplings_than_the_accumulators_hold():
    """The 56-bit accumulators are proven not to overflow up to 146 couplings per site; the form takes
    at most 127 (plus the on-site term)."""
    sc = bcc_two_site(L=32)
    assert fixed_point_eligible(sc)
    many = bcc_two_site(L=32)
    many.bond_src = np.zeros(128, np.int32)
    assert not fixed_point_eligible(many)
