/* empty stand-in (TEST INFRASTRUCTURE ONLY) */
