// empty: the reference configure step would generate this file
