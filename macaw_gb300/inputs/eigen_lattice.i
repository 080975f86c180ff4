# k-eigenvalue pin lattice: the 17x17 lattice (2,039,184 tets) with every
# fuel nuclide fissionable (nu*sigma_f = 2.43 * 0.6 * sigma_a), constant
# scattering (2 b) and absorption (0.5 b) added to the synthetic tables,
# reflective sides, vacuum top and bottom; 1e6 particles per generation,
# 3 inactive and 10 active generations (OpenMC run_mode eigenvalue).
[Mesh]
  [lattice]
    type = TetLatticeMeshGenerator
    nx = 17
    ny = 17
    nz = 21
    pitch = 1.26
    height = 50
  []
[]

[RayKernels/collision]
  type = CollisionKernel
  temperature = temperature
  blocks = '1 2 3'
  materials = '1 2 3'
[]

[RayBCs]
  [sides]
    type = ReflectRayBC
    boundary = 'right left top bottom'
  []
  [ends]
    type = KillRayBC
    boundary = 'back front'
  []
[]

[UserObjects]
  [xs]
    type = SyntheticCrossSections
    material_ids = '1 2 3'
    nuclides_per_material = '15 4 3'
    n_points = 20000
    scattering_offset = 2
    absorption_offset = 0.5
    fissionable_materials = '1'
    nu = 2.43
    fission_share = 0.6
  []
  [study]
    type = OpenMCStudy
    run_mode = eigenvalue
    particles = 1000000
    inactive = 3
    bank_size = 1000000
    source_space = cylinders
    precision = fp64
  []
  [pintally]
    type = OpenMCTally
    id = 1
    estimator = TRACKLENGTH
    scores = 'flux'
    filters = 'cell'
  []
[]

[AuxKernels]
  [cell_flux]
    type = OpenMCTallyAux
    tally_id = 1
    granularity = cell
    score = flux
    variable = flux
  []
[]

[Executioner]
  type = Transient
  num_steps = 13
[]

[Outputs]
  csv = true
[]
