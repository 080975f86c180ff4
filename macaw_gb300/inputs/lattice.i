# 17x17 pin lattice, pitch 1.26 cm, 50 cm tall (2,039,184 tets): fuel,
# clad and moderator with 15/4/3 synthetic nuclides on 20,000-point grids,
# uniform source in the fuel cylinders, 10 batches of 1e6 histories.
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
  [vacuum]
    type = KillRayBC
    boundary = 'back front top right left bottom'
  []
[]

[UserObjects]
  [xs]
    type = SyntheticCrossSections
    material_ids = '1 2 3'
    nuclides_per_material = '15 4 3'
    n_points = 20000
  []
  [study]
    type = OpenMCStudy
    particles = 1000000
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
  [blocktally]
    type = OpenMCTally
    id = 2
    estimator = TRACKLENGTH
    scores = 'flux'
    filters = 'universe'
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
  [block_flux]
    type = OpenMCTallyAux
    tally_id = 2
    granularity = universe
    score = flux
    variable = block_flux
  []
[]

[Executioner]
  type = Transient
  num_steps = 10
[]
