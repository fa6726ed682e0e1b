//! The crate's own iterative integration tests (src/tests/fem/test_fem.rs:83-225), run through this
//! facade: a 2-node truss along x (E = 1e6, A = 2, L = 30), node 1 held in X, 100 along X at node 2.
//! Known answers: u2x = PL/EA = 0.0015 (the crate's f32 test prints 0.0014999999), the reaction at node 1
//! -100, the truss's axial force 100, one PCG iteration.  Here in f64, so the values are compared to
//! 1e-12 relative.  The one call the crate does not make: `assemble`, since the crate assembles inside
//! every `add_*` and this library builds the stiffness in one GPU pass.  Needs a CUDA device and the
//! built library (`cargo test` after `python -m finite_element_method_gb300.build`).

use finite_element_method_gb300::{DOFParameter, ElementForceComponent, FEM};

fn close(got: f64, want: f64) -> bool {
    (got - want).abs() <= 1e-12 * want.abs().max(1.0)
}

fn truss_model() -> Result<FEM, String> {
    let mut model = FEM::create(1e-4, 1e-12, 2);
    model.add_node(1, 0.0, 0.0, 0.0)?;
    model.add_node(2, 30.0, 0.0, 0.0)?;
    model.add_truss(1, 1, 2, 1e6, 2.0, None)?;
    model.add_displacement(1, DOFParameter::X, 0.0)?;
    model.add_concentrated_load(2, DOFParameter::X, 100.0)?;
    model.assemble()?;
    Ok(model)
}

fn solve_and_check(block_jacobi: bool) -> Result<(), String> {
    let mut model = truss_model()?;
    let sep = model.separate_stiffness_matrix_sparse_iterative()?;
    let r_a_vector = model.compose_r_a_vector(sep.get_k_aa_indexes())?;
    let u_b_vector = model.compose_u_b_vector(sep.get_k_bb_indexes())?;
    let (u_a_vector, iterations) = if block_jacobi {
        model.find_ua_vector_iterative_pcg_block_jacobi_sparse(&sep, &r_a_vector, &u_b_vector, 1000)?
    } else {
        model.find_ua_vector_iterative_pcg_jacobi_sparse(&sep, &r_a_vector, &u_b_vector, 1000)?
    };
    let r_r_vector = model.find_r_r_vector_sparse(&sep, &u_a_vector, &u_b_vector)?;
    model.compose_global_analysis_result(sep.get_k_aa_indexes(), sep.get_k_bb_indexes(), &u_a_vector, &r_r_vector)?;

    let mut global = model.extract_global_analysis_result()?;
    global.sort_by(|a, b| (a.0, a.1).cmp(&(b.0, b.1)));
    let mut expected = Vec::new();
    for node in [1u32, 2] {
        for p in 0..6 {
            let dof = DOFParameter::from_usize(p);
            let (u, f) = match (node, dof) {
                (1, DOFParameter::X) => (0.0, -100.0),
                (2, DOFParameter::X) => (0.0015, 100.0),
                _ => (0.0, 0.0),
            };
            expected.push((node, dof, u, f));
        }
    }
    assert_eq!(global.len(), expected.len());
    for (g, e) in global.iter().zip(expected.iter()) {
        assert_eq!((g.0, g.1), (e.0, e.1));
        assert!(close(g.2, e.2) && close(g.3, e.3), "{g:?} against {e:?}");
    }

    let elements = model.extract_elements_analysis_result()?;
    assert_eq!(elements.len(), 1);
    assert_eq!(elements[0].0, 1);
    assert_eq!(elements[0].1.len(), 1);
    assert_eq!(elements[0].1[0].0, ElementForceComponent::ForceR);
    assert!(close(elements[0].1[0].1, 100.0), "{:?}", elements[0]);
    assert_eq!(iterations, 1);
    Ok(())
}

#[test]
fn test_integration_iterative_pcg_jacobi_sparse() -> Result<(), String> {
    solve_and_check(false)
}

#[test]
fn test_integration_iterative_pcg_block_jacobi_sparse() -> Result<(), String> {
    solve_and_check(true)
}

#[test]
fn test_sparse_separation_truss_has_kaa() -> Result<(), String> {
    let model = truss_model()?;
    let sep = model.separate_stiffness_matrix_sparse_iterative()?;
    assert!(sep.get_n_aa() > 0);
    assert!(!sep.get_k_aa_triplets().is_empty());
    Ok(())
}

#[test]
fn test_stiffness_of_the_truss() -> Result<(), String> {
    // EA/L on the X DOFs of the two nodes (0 and 6), nothing else stored
    let model = truss_model()?;
    let csr = model.stiffness_csr()?;
    let k = 1e6 * 2.0 / 30.0;
    let mut entries = Vec::new();
    for r in 0..csr.row_ptr.len() - 1 {
        for q in csr.row_ptr[r] as usize..csr.row_ptr[r + 1] as usize {
            entries.push((r, csr.col_idx[q] as usize, csr.values[q]));
        }
    }
    let want = [(0, 0, k), (0, 6, -k), (6, 0, -k), (6, 6, k)];
    assert_eq!(entries.len(), want.len(), "{entries:?}");
    for (g, w) in entries.iter().zip(want.iter()) {
        assert_eq!((g.0, g.1), (w.0, w.1));
        assert!(close(g.2, w.2), "{g:?} against {w:?}");
    }
    Ok(())
}
