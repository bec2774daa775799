"""rvgp_gb300: the RVGP numerical core as hand-written CUDA kernels for GB300 (sm_103a).

Drop-in names of the reference package (RVGP/__init__.py:1-3)::

    import rvgp_gb300 as RVGP
    d = RVGP.create_data_object(X, n_eigenpairs=50)
    d.random_vector_field(seed=1); d.smooth_vector_field(t=100)
    gp = RVGP.fit(d, train_ind=train_ind)
    mean, var = gp.transform(d, test_ind)
"""
from rvgp_gb300 import kernels  # noqa: F401
from rvgp_gb300.dataclass import data as create_data_object  # noqa: F401
from rvgp_gb300.dataclass import load_data_object  # noqa: F401
from rvgp_gb300.main import train_gp as fit  # noqa: F401
