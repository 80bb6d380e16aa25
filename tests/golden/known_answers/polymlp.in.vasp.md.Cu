n_type 1
elements Cu

feature_type gtinv
cutoff 8.0
model_type 3
max_p 2

gtinv_order 3
gtinv_maxl 4 4

gaussian_params1 1.0 1.0 1
gaussian_params2 0.0 7.0 8

reg_alpha_params -3 1 5

atomic_energy -0.00040000

data_md data-vasp-md-Cu/vasprun.xml

include_stress False
gtinv_version 1
