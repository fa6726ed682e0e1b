//! A batch of recorded call sequences ([`Structures`] -> [`Batch::from_calls`]) gives every structure the
//! CSR its own plain sequence (`FEM::create`, `add_*`, `assemble`) gives, bit for bit.  Needs a CUDA device
//! and the built library.

use finite_element_method_gb300::{Batch, BeamSection, FEM, Structures};

enum Call {
    Node(u32, [f64; 3]),
    Truss(u32, [u32; 2], f64, f64),
    Beam(u32, [u32; 2], BeamSection),
    Plate(u32, [u32; 4], [f64; 4]),
}

fn section(axis: [f64; 3]) -> BeamSection {
    BeamSection {
        young_modulus: 210e9,
        poisson_ratio: 0.3,
        area: 1.2e-2,
        i11: 8e-5,
        i22: 3e-5,
        i12: 0.0,
        it: 2e-5,
        shear_factor: 5.0 / 6.0,
        local_axis_1_direction: axis,
    }
}

/// (nodes_number, calls) of each structure: a truss; a slab of one plate with a column under a corner; a
/// beam with room for more nodes than it adds
fn sequences() -> Vec<(u32, Vec<Call>)> {
    let plate = [70e9, 0.3, 0.02, 5.0 / 6.0];
    vec![
        (2, vec![Call::Node(1, [0.0, 0.0, 0.0]), Call::Node(2, [30.0, 0.0, 0.0]), Call::Truss(1, [1, 2], 1e6, 2.0)]),
        (
            5,
            vec![
                Call::Node(1, [1.0, 1.0, 3.0]),
                Call::Node(2, [0.0, 1.0, 3.0]),
                Call::Node(3, [0.0, 0.0, 3.0]),
                Call::Node(4, [1.0, 0.0, 3.0]),
                Call::Node(5, [1.0, 1.0, 0.0]),
                Call::Beam(1, [5, 1], section([1.0, 0.0, 0.0])),
                Call::Plate(1, [1, 2, 3, 4], plate),
            ],
        ),
        (4, vec![Call::Node(7, [0.0, 0.0, 0.0]), Call::Node(9, [3.0, 0.5, 0.2]), Call::Beam(3, [7, 9], section([0.0, 0.0, 1.0]))]),
    ]
}

#[test]
fn batch_matches_plain_sequences() -> Result<(), String> {
    let mut rec = Structures::new();
    let mut plain = Vec::new();
    for (nodes_number, calls) in sequences() {
        rec.create(nodes_number);
        let mut model = FEM::create(1e-12, 1e-12, nodes_number);
        for call in &calls {
            match call {
                Call::Node(n, x) => {
                    rec.add_node(*n, x[0], x[1], x[2]);
                    model.add_node(*n, x[0], x[1], x[2])?;
                }
                Call::Truss(n, nodes, e, a) => {
                    rec.add_truss(*n, nodes[0], nodes[1], *e, *a, None);
                    model.add_truss(*n, nodes[0], nodes[1], *e, *a, None)?;
                }
                Call::Beam(n, nodes, s) => {
                    rec.add_beam(*n, nodes[0], nodes[1], s);
                    model.add_beam(
                        *n,
                        nodes[0],
                        nodes[1],
                        s.young_modulus,
                        s.poisson_ratio,
                        s.area,
                        s.i11,
                        s.i22,
                        s.i12,
                        s.it,
                        s.shear_factor,
                        s.local_axis_1_direction,
                    )?;
                }
                Call::Plate(n, nodes, p) => {
                    rec.add_plate(*n, nodes[0], nodes[1], nodes[2], nodes[3], p[0], p[1], p[2], p[3]);
                    model.add_plate(*n, nodes[0], nodes[1], nodes[2], nodes[3], p[0], p[1], p[2], p[3])?;
                }
            }
        }
        model.assemble()?;
        plain.push(model.stiffness_csr()?);
    }
    let batch = Batch::from_calls(1e-12, 1e-12, &mut rec)?;
    assert_eq!(batch.len(), plain.len());
    for (i, want) in plain.iter().enumerate() {
        let got = batch.csr(i)?;
        assert_eq!(got.row_ptr, want.row_ptr, "structure {i}");
        assert_eq!(got.col_idx, want.col_idx, "structure {i}");
        assert_eq!(got.values.len(), want.values.len());
        assert!(got.values.iter().zip(&want.values).all(|(a, b)| a.to_bits() == b.to_bits()), "structure {i}");
    }
    Ok(())
}
