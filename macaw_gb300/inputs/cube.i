# Fixed-source point source in the 20 cm cube of 20^3 hexes x 6 tets
# (48,000 tets), one material of 10 synthetic nuclides, vacuum boundary.
[Mesh]
  [cube]
    type = TetCubeMeshGenerator
    n = 20
    length = 20
  []
[]

[Variables/temperature]
  order = CONSTANT
  family = MONOMIAL
[]

[AuxVariables/flux]
  order = CONSTANT
  family = MONOMIAL
[]

[RayKernels/collision]
  type = CollisionKernel
  temperature = temperature
  blocks = '0'
  materials = '1'
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
    material_ids = '1'
    nuclides_per_material = '10'
    n_points = 10000
    seed = 20240611
  []
  [study]
    type = OpenMCStudy
    particles = 100000
    source_space = point
    source_point = '10 10 10'
    execute_on = TIMESTEP_END
  []
  [celltally]
    type = OpenMCTally
    id = 1
    particle_type = 'neutron'
    estimator = 'TRACKLENGTH'
    scores = 'flux'
    filters = 'cell'
    execute_on = 'initial'
  []
[]

[AuxKernels]
  [cell_val]
    type = OpenMCTallyAux
    tally_id = 1
    granularity = cell
    estimator = TRACKLENGTH
    particle_type = neutron
    score = 'flux'
    variable = flux
    execute_on = TIMESTEP_END
  []
[]

[Executioner]
  type = Transient
  num_steps = 1
[]

[Outputs]
  csv = true
[]
