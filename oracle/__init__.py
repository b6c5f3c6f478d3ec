"""CPU oracle for the fd2dmpi hot path -- test infrastructure, never the product."""
